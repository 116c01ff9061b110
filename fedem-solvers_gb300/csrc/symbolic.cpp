// symbolic.cpp -- ordering and symbolic factorisation for the multifrontal
// LDL^T of the Newton matrix.
//
// This replaces the symbolic phase of the SAM/SPR sparse solver that the
// reference calls through csAllocPointerArrays / csRenumber / csPreassemble
// (src/vpmCommon/vpmLinAlg/asmExtensionModule.f90:227-893: SPRPRP, SPRSAS,
// SPRRNM, SPRTRS, SPRSMB).  SPR's source is not part of the reference tree,
// so the ordering here is our own, deterministic and documented:
//   * equations are grouped by triad, by part and by joint (all free DOFs of a
//     triad, the free generalized DOFs of a part, or all free DOFs of a joint,
//     form one node); nodes are adjacent when the Newton matrix pattern couples
//     them;
//   * nested dissection on the node graph: breadth-first level structures
//     from a pseudo-peripheral node, the separator is the smallest level set
//     in the middle third; components of at most LEAF_NODES nodes are leaves;
//   * every separator and every leaf is one supernode (front); supernodes are
//     eliminated in post-order of the dissection tree;
//   * the assembly tree parent of a front is the front owning the first
//     (lowest-position) row of its update set.
// Fronts of equal height (distance from the leaves) are independent, which is
// what lets the GPU factor and solve level by level across all models.

#include <algorithm>
#include <cstring>
#include <numeric>

#include "host_model.h"

namespace fgpu {

namespace {
const int LEAF_NODES = 3;

struct NodeGraph {
  int n = 0;
  std::vector<int> adjPtr, adj;     // node adjacency (CSR)
  std::vector<int> eqPtr, eqs;      // free equations of each node, DOF order
};

// BFS over the nodes of one component (mark == tag); returns the order and levels.
void bfs(const NodeGraph& g, int start, const std::vector<int>& mark, int tag, std::vector<int>& order,
         std::vector<int>& level, std::vector<int>& levelOf) {
  order.clear();
  level.clear();
  order.push_back(start);
  levelOf[start] = 0;
  size_t head = 0;
  int curLevel = -1;
  while (head < order.size()) {
    int v = order[head++];
    if (levelOf[v] != curLevel) { curLevel = levelOf[v]; level.push_back((int)head - 1); }
    for (int k = g.adjPtr[v]; k < g.adjPtr[v + 1]; ++k) {
      int w = g.adj[k];
      if (mark[w] != tag || levelOf[w] >= 0) continue;
      levelOf[w] = levelOf[v] + 1;
      order.push_back(w);
    }
  }
  level.push_back((int)order.size());
}

}  // namespace

int symbolicAnalysis(HostModel& m, std::string& err) {
  // ---- node graph -------------------------------------------------------
  // nodes: the free equations of each triad, then of each joint (DOF order);
  // two nodes are adjacent when the Newton matrix couples their equations
  NodeGraph g;
  std::vector<int> eqNode(m.neq, -1);
  g.eqPtr.assign(1, 0);
  auto addNode = [&](int d0, int nd) {
    bool any = false;
    for (int d = d0; d < d0 + nd; ++d)
      if (m.meqn[d] >= 0) {
        eqNode[m.meqn[d]] = g.n;
        g.eqs.push_back(m.meqn[d]);
        any = true;
      }
    if (any) {
      g.eqPtr.push_back((int)g.eqs.size());
      ++g.n;
    }
  };
  for (int t = 0; t < m.ntri; ++t) addNode(m.triFirstDof[t], m.triNdof[t]);
  for (int p = 0; p < m.npart; ++p) addNode(m.pGenFirstDof[p], m.pNgen[p]);  // a part's generalized DOFs
  for (int j = 0; j < m.njoint; ++j) addNode(m.jFirstDof[j], m.jNdof[j]);
  for (int e = 0; e < m.neq; ++e)
    if (eqNode[e] < 0) { err = "equation without a node"; return -43; }
  std::vector<std::vector<int>> nb(g.n);
  for (int i = 0; i < m.neq; ++i)
    for (int k = m.rowPtr[i]; k < m.rowPtr[i + 1]; ++k) {
      const int a = eqNode[i], b = eqNode[m.colInd[k]];
      if (a != b) nb[a].push_back(b);
    }
  g.adjPtr.assign(g.n + 1, 0);
  for (int v = 0; v < g.n; ++v) {
    std::sort(nb[v].begin(), nb[v].end());
    nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
    g.adjPtr[v + 1] = g.adjPtr[v] + (int)nb[v].size();
    g.adj.insert(g.adj.end(), nb[v].begin(), nb[v].end());
  }

  // ---- nested dissection ---------------------------------------------------
  struct SNode { std::vector<int> nodes; int ndParent; };
  std::vector<SNode> sn;
  struct Task { std::vector<int> nodes; int parent; };
  std::vector<Task> stack;
  {
    std::vector<int> all(g.n);
    std::iota(all.begin(), all.end(), 0);
    stack.push_back({all, -1});
  }
  std::vector<int> mark(g.n, -1), levelOf(g.n, -1), order, level;
  int tagCounter = 0;
  while (!stack.empty()) {
    Task task = std::move(stack.back());
    stack.pop_back();
    int tag = tagCounter++;
    for (int v : task.nodes) mark[v] = tag;
    // connected components in the order of their lowest node
    std::vector<int> sortedNodes = task.nodes;
    std::sort(sortedNodes.begin(), sortedNodes.end());
    for (int s : sortedNodes) {
      if (mark[s] != tag || levelOf[s] >= 0) continue;
      bfs(g, s, mark, tag, order, level, levelOf);
      std::vector<int> comp = order;
      int ctag = tagCounter++;
      for (int v : comp) { mark[v] = ctag; levelOf[v] = -1; }
      if ((int)comp.size() <= LEAF_NODES) {
        std::sort(comp.begin(), comp.end());
        sn.push_back({comp, task.parent});
        for (int v : comp) mark[v] = -2;
        continue;
      }
      // pseudo-peripheral start: repeat BFS from the farthest node while the depth grows
      int start = *std::min_element(comp.begin(), comp.end());
      int depth = -1;
      for (int it = 0; it < 4; ++it) {
        bfs(g, start, mark, ctag, order, level, levelOf);
        int d = (int)level.size() - 1;
        int far = order.back();
        for (int v : order) levelOf[v] = -1;
        if (d <= depth) break;
        depth = d;
        // among the last level pick the lowest node number (deterministic)
        int best = far;
        for (int k = level[level.size() - 2]; k < level.back(); ++k) best = std::min(best, order[k]);
        start = best;
      }
      bfs(g, start, mark, ctag, order, level, levelOf);
      int nlev = (int)level.size() - 1;
      if (nlev < 3) {
        std::vector<int> c2 = order;
        for (int v : c2) levelOf[v] = -1;
        std::sort(c2.begin(), c2.end());
        sn.push_back({c2, task.parent});
        for (int v : c2) mark[v] = -2;
        continue;
      }
      int lo = std::max(1, nlev / 3), hi = std::min(nlev - 2, (2 * nlev) / 3);
      int mid = nlev / 2, best = mid;
      for (int l = lo; l <= hi; ++l) {
        int sz = level[l + 1] - level[l], bsz = level[best + 1] - level[best];
        if (sz < bsz || (sz == bsz && std::abs(l - mid) < std::abs(best - mid))) best = l;
      }
      std::vector<int> sep(order.begin() + level[best], order.begin() + level[best + 1]);
      std::vector<int> rest;
      for (int k = 0; k < (int)order.size(); ++k)
        if (k < level[best] || k >= level[best + 1]) rest.push_back(order[k]);
      for (int v : order) levelOf[v] = -1;
      std::sort(sep.begin(), sep.end());
      int sid = (int)sn.size();
      sn.push_back({sep, task.parent});
      for (int v : sep) mark[v] = -2;
      stack.push_back({rest, sid});
    }
  }

  // ---- post-order of the dissection tree -> elimination positions -----------
  int nsn = (int)sn.size();
  std::vector<std::vector<int>> ndChildren(nsn);
  std::vector<int> roots;
  for (int s = 0; s < nsn; ++s) {
    if (sn[s].ndParent < 0) roots.push_back(s);
    else ndChildren[sn[s].ndParent].push_back(s);
  }
  std::vector<int> post;
  post.reserve(nsn);
  {
    std::vector<std::pair<int, int>> st;
    for (int r : roots) {
      st.push_back({r, 0});
      while (!st.empty()) {
        auto& top = st.back();
        if (top.second < (int)ndChildren[top.first].size()) {
          int c = ndChildren[top.first][top.second++];
          st.push_back({c, 0});
        } else {
          post.push_back(top.first);
          st.pop_back();
        }
      }
    }
  }
  std::vector<int> pos(m.neq, -1);
  m.perm.assign(m.neq, -1);
  std::vector<int> frontOfPos(m.neq, -1), pivStart(nsn), pivEnd(nsn);
  int p = 0;
  for (int f = 0; f < nsn; ++f) {
    const SNode& s = sn[post[f]];
    pivStart[f] = p;
    for (int v : s.nodes)
      for (int k = g.eqPtr[v]; k < g.eqPtr[v + 1]; ++k) {
        pos[g.eqs[k]] = p;
        m.perm[p] = g.eqs[k];
        frontOfPos[p] = f;
        ++p;
      }
    pivEnd[f] = p;
  }
  if (p != m.neq) { err = "symbolic analysis lost equations"; return -40; }

  // ---- fronts: update sets, assembly tree, maps ---------------------------------
  m.fronts.assign(nsn, Front());
  std::vector<std::vector<int>> upd(nsn);  // update rows as positions, sorted
  std::vector<std::vector<int>> children(nsn);
  std::vector<int> mark2(m.neq, -1);
  for (int f = 0; f < nsn; ++f) {
    std::vector<int> rows;
    for (int q = pivStart[f]; q < pivEnd[f]; ++q) {
      int eq = m.perm[q];
      for (int k = m.rowPtr[eq]; k < m.rowPtr[eq + 1]; ++k) {
        int pq = pos[m.colInd[k]];
        if (pq >= pivEnd[f] && mark2[pq] != f) { mark2[pq] = f; rows.push_back(pq); }
      }
    }
    for (int c : children[f])
      for (int pq : upd[c])
        if (pq >= pivEnd[f] && mark2[pq] != f) { mark2[pq] = f; rows.push_back(pq); }
    std::sort(rows.begin(), rows.end());
    upd[f] = rows;
    Front& fr = m.fronts[f];
    fr.npiv = pivEnd[f] - pivStart[f];
    fr.nrow = fr.npiv + (int)rows.size();
    fr.parent = rows.empty() ? -1 : frontOfPos[rows[0]];
    if (fr.parent >= 0) children[fr.parent].push_back(f);
  }
  int64_t rowOff = 0, lOff = 0, uOff = 0, wOff = 0, childOff = 0, relOff = 0, asmOff = 0;
  m.maxHeight = 0;
  m.maxFront = 0;
  for (int f = 0; f < nsn; ++f) {
    Front& fr = m.fronts[f];
    fr.height = 0;
    for (int c : children[f]) fr.height = std::max(fr.height, m.fronts[c].height + 1);
    m.maxHeight = std::max(m.maxHeight, fr.height);
    m.maxFront = std::max(m.maxFront, fr.nrow);
    int u = fr.nrow - fr.npiv;
    fr.rowOff = rowOff;
    fr.lOff = lOff;
    fr.uOff = uOff;
    fr.wOff = wOff;
    fr.childOff = childOff;
    fr.nchild = (int)children[f].size();
    fr.relOff = relOff;
    rowOff += fr.nrow;
    lOff += (int64_t)fr.nrow * fr.npiv;
    uOff += (int64_t)u * u;
    wOff += u;
    childOff += fr.nchild;
    relOff += u;
    for (int q = pivStart[f]; q < pivEnd[f]; ++q) m.frontRows.push_back(m.perm[q]);
    for (int pq : upd[f]) m.frontRows.push_back(m.perm[pq]);
    m.childList.insert(m.childList.end(), children[f].begin(), children[f].end());
  }
  m.lSize = lOff;
  m.uSize = uOff;
  m.wSize = wOff;
  // relative indices of each update row inside the parent front
  m.relIndex.assign(relOff, -1);
  for (int f = 0; f < nsn; ++f) {
    const Front& fr = m.fronts[f];
    if (fr.parent < 0) continue;
    const Front& pa = m.fronts[fr.parent];
    const int* prow = &m.frontRows[pa.rowOff];
    for (int k = 0; k < fr.nrow - fr.npiv; ++k) {
      int target = pos[m.frontRows[fr.rowOff + fr.npiv + k]];
      int idx = -1;
      // parent rows are sorted by position: pivots first then update rows
      int lo = 0, hi = pa.nrow - 1;
      while (lo <= hi) {
        int mid = (lo + hi) / 2;
        int pm = pos[prow[mid]];
        if (pm < target) lo = mid + 1;
        else if (pm > target) hi = mid - 1;
        else { idx = mid; break; }
      }
      if (idx < 0) { err = "inconsistent assembly tree"; return -41; }
      m.relIndex[fr.relOff + k] = idx;
    }
  }
  // original matrix entries of the pivot columns: (CSR slot, column-major front index)
  for (int f = 0; f < nsn; ++f) {
    Front& fr = m.fronts[f];
    fr.asmOff = asmOff;
    const int* rowsF = &m.frontRows[fr.rowOff];
    for (int cj = 0; cj < fr.npiv; ++cj) {
      int eq = rowsF[cj];
      int pj = pos[eq];
      for (int k = m.rowPtr[eq]; k < m.rowPtr[eq + 1]; ++k) {
        int pi = pos[m.colInd[k]];
        if (pi < pj) continue;
        int lo = 0, hi = fr.nrow - 1, idx = -1;
        while (lo <= hi) {
          int mid = (lo + hi) / 2;
          int pm = pos[rowsF[mid]];
          if (pm < pi) lo = mid + 1;
          else if (pm > pi) hi = mid - 1;
          else { idx = mid; break; }
        }
        if (idx < 0) { err = "matrix entry outside its front"; return -42; }
        m.asmSlot.push_back(k);
        m.asmPos.push_back(idx + fr.nrow * cj);
      }
    }
    fr.nasm = (int)(m.asmSlot.size() - asmOff);
    asmOff = (int64_t)m.asmSlot.size();
  }
  return 0;
}

}  // namespace fgpu
