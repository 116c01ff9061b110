// eigen.cpp -- lowest eigenmodes of K phi = lambda M phi at the current state.
//
// Replaces the eigenvalue analysis the reference runs through SAM's Lanczos
// solver (src/vpmSolver/modesRoutinesModule.f90:649-942, csLanczosEigenSolve;
// solverModule.f90:1004-1092 returns sqrt|lambda| / 2 pi).  Here: Lanczos-type
// iteration on the shift-invert operator K^-1 M (shift 0) in the M inner
// product: a block Krylov space (block size 3, so that repeated eigenvalues --
// the two bending planes of a symmetric section -- are found) with full
// reorthogonalisation, and Rayleigh-Ritz on the projected matrix, whose
// eigenpairs come from the cyclic Jacobi method.  Every K^-1 application is one
// solve with the stiffness matrix factored once on the GPU by the multifrontal
// kernels (FP64 refinement in mixed precision); M v is formed on the host from
// the element mass matrices in their current frames.

#include "eigen.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace fgpu {
namespace {

// eigenvalues (ascending) and eigenvectors (column-major n x n, in the order
// of the values) of the symmetric matrix H (column-major n x n) by the cyclic
// Jacobi method: plane rotations that zero one off-diagonal pair at a time,
// swept until the off-diagonal part is negligible
void jacobiEigen(std::vector<double> H, int n, std::vector<double>& val, std::vector<double>& vec) {
  auto h = [&](int i, int j) -> double& { return H[(size_t)i + (size_t)n * j]; };
  std::vector<double> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i + (size_t)n * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < n; ++j) {
      diag += h(j, j) * h(j, j);
      for (int i = 0; i < j; ++i) off += h(i, j) * h(i, j);
    }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double hpq = h(p, q);
        if (hpq == 0.0) continue;
        // rotation angle: tan(2 phi) = 2 h_pq / (h_qq - h_pp), the smaller root for t = tan(phi)
        const double theta = (h(q, q) - h(p, p)) / (2.0 * hpq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double hkp = h(k, p), hkq = h(k, q);
          h(k, p) = c * hkp - s * hkq;
          h(k, q) = s * hkp + c * hkq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double hpk = h(p, k), hqk = h(q, k);
          h(p, k) = c * hpk - s * hqk;
          h(q, k) = s * hpk + c * hqk;
        }
        for (int k = 0; k < n; ++k) {
          double& vp = V[(size_t)k + (size_t)n * p];
          double& vq = V[(size_t)k + (size_t)n * q];
          const double a = vp, b = vq;
          vp = c * a - s * b;
          vq = s * a + c * b;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return h(a, a) < h(b, b); });
  val.resize(n);
  vec.assign((size_t)n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    val[k] = h(idx[k], idx[k]);
    for (int i = 0; i < n; ++i) vec[(size_t)i + (size_t)n * k] = V[(size_t)i + (size_t)n * idx[k]];
  }
}

double dot(const std::vector<double>& a, const double* b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
double dotp(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

}  // namespace

// mass matrix of model 0 over the free equations in CSR (the model's pattern):
// element mass matrices rotated with the current frames (addInSysModule.f90
// BuildMassMat semantics); axial springs and dampers carry no mass
void massCsr(const HostModel& m, const std::vector<double>& frames, std::vector<double>& vals) {
  vals.assign(m.colInd.size(), 0.0);
  auto slot = [&](int i, int j) {
    const int* b = m.colInd.data() + m.rowPtr[i];
    const int* e = m.colInd.data() + m.rowPtr[i + 1];
    const int* p = std::lower_bound(b, e, j);
    return (p != e && *p == j) ? (int)(p - m.colInd.data()) : -1;
  };
  for (int el = 0; el < m.nel; ++el) {
    const double* X = &m.M[144 * (size_t)el];
    const double* R = &frames[12 * (size_t)el];
    const int* q = &m.elEq[12 * (size_t)el];
    for (int bj = 0; bj < 4; ++bj)
      for (int bi = 0; bi < 4; ++bi) {
        double W[9];
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) {
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += R[r + 3 * k] * X[(3 * bi + k) + 12 * (3 * bj + c)];
            W[r + 3 * c] = v;
          }
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) {
            const int i = q[3 * bi + r], j = q[3 * bj + c];
            if (i < 0 || j < 0) continue;
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += W[r + 3 * k] * R[c + 3 * k];
            const int s = slot(i, j);
            if (s >= 0) vals[s] += v;
          }
      }
  }
}

int lowestModes(Engine& eng, const HostModel& m, int nmod, std::vector<double>& lambda, std::vector<double>& vecs,
                int& nNeg) {
  const int n = m.neq;
  if (nmod < 1 || nmod > n) return -1;
  std::vector<double> frames(12 * (size_t)m.nel), Mv;
  eng.getElementFrames(0, frames.data());
  massCsr(m, frames, Mv);
  auto massTimes = [&](const double* x, double* y) {
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = m.rowPtr[i]; k < m.rowPtr[i + 1]; ++k) s += Mv[k] * x[m.colInd[k]];
      y[i] = s;
    }
  };
  int rc = eng.prepareStiffnessSolves();
  if (rc) {
    eng.endStiffnessSolves();
    return rc;
  }
  // K x = b to FP64 accuracy: the GPU solve (FP32 fronts with refinement in
  // mixed precision, FP64 otherwise), then iterative refinement against the
  // FP64 stiffness matrix (its CSR values from the assembly) -- K alone is far
  // worse conditioned than a dynamic Newton matrix
  std::vector<double> Kv(m.colInd.size()), res(n), dx(n);
  eng.getCsrValues(0, Kv.data());
  auto solveK = [&](const double* bvec, double* x) {
    int r2 = eng.solveStiffness(0, bvec, x);
    double bn = 0.0;
    for (int i = 0; i < n; ++i) bn = std::max(bn, std::fabs(bvec[i]));
    for (int it = 0; it < 40 && r2 == 0; ++it) {
      double rn = 0.0;
      for (int i = 0; i < n; ++i) {
        double s2 = bvec[i];
        for (int k = m.rowPtr[i]; k < m.rowPtr[i + 1]; ++k) s2 -= Kv[k] * x[m.colInd[k]];
        res[i] = s2;
        rn = std::max(rn, std::fabs(s2));
      }
      if (rn <= 1e-14 * bn) break;
      r2 = eng.solveStiffness(0, res.data(), dx.data());
      for (int i = 0; i < n; ++i) x[i] += dx[i];
    }
    return r2;
  };
  // block Krylov space of K^-1 M (block size b: repeated eigenvalues up to
  // multiplicity b are found), M-orthonormal basis Q with A Q kept, Rayleigh-Ritz
  // on H = (M Q)^T (A Q)
  const int b = std::min(3, n);
  const int mMax = std::min(n, std::max(4 * nmod + 24, 60));
  std::vector<double> Q, AQ, MQ;
  Q.reserve((size_t)n * mMax);
  std::vector<double> w(n), mw(n);
  uint64_t seed = 0x9e3779b97f4a7c15ull;
  auto addVector = [&](std::vector<double>& v) {  // M-orthogonalise against Q (twice), normalise, append
    const int cols = (int)(Q.size() / n);
    massTimes(v.data(), mw.data());
    const double nv0 = std::sqrt(std::max(dot(v, mw.data()), 0.0));
    for (int pass = 0; pass < 2; ++pass) {
      massTimes(v.data(), mw.data());
      for (int k = 0; k < cols; ++k) {
        const double* qk = &Q[(size_t)n * k];
        const double c = dot(mw, qk);
        for (int i = 0; i < n; ++i) v[i] -= c * qk[i];
      }
    }
    massTimes(v.data(), mw.data());
    const double nv = std::sqrt(std::max(dot(v, mw.data()), 0.0));
    if (!(nv > 1e-10 * nv0)) return false;  // no new direction
    for (int i = 0; i < n; ++i) v[i] /= nv;
    Q.insert(Q.end(), v.begin(), v.end());
    massTimes(v.data(), mw.data());
    MQ.insert(MQ.end(), mw.begin(), mw.end());
    return true;
  };
  for (int k = 0; k < b; ++k) {
    for (int i = 0; i < n; ++i) {
      seed = seed * 6364136223846793005ull + 1442695040888963407ull;
      w[i] = (double)(seed >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    addVector(w);
  }
  std::vector<double> theta, Y;
  bool converged = false;
  int done = 0;  // basis vectors with A q computed
  while (!converged && rc == 0) {
    const int cols = (int)(Q.size() / n);
    // A q for the newest block, then the next block from it
    std::vector<std::vector<double>> next;
    for (int k = done; k < cols; ++k) {
      rc = solveK(&MQ[(size_t)n * k], w.data());
      if (rc) break;
      AQ.insert(AQ.end(), w.begin(), w.end());
      next.push_back(w);
    }
    if (rc) break;
    done = cols;
    // Rayleigh-Ritz on the current basis
    std::vector<double> H((size_t)cols * cols);
    for (int j = 0; j < cols; ++j)
      for (int i = 0; i <= j; ++i) {
        const double hij = 0.5 * (dotp(&MQ[(size_t)n * i], &AQ[(size_t)n * j], n) +
                                  dotp(&MQ[(size_t)n * j], &AQ[(size_t)n * i], n));
        H[(size_t)i + (size_t)cols * j] = H[(size_t)j + (size_t)cols * i] = hij;
      }
    jacobiEigen(H, cols, theta, Y);
    if (cols >= nmod) {
      // residuals of the nmod largest Ritz pairs: A x - theta x with x = Q y
      converged = true;
      for (int k = 0; k < nmod && converged; ++k) {
        const int col = cols - 1 - k;
        std::vector<double> r(n, 0.0);
        for (int s2 = 0; s2 < cols; ++s2) {
          const double y = Y[(size_t)s2 + (size_t)cols * col];
          const double* aq = &AQ[(size_t)n * s2];
          const double* q = &Q[(size_t)n * s2];
          for (int i = 0; i < n; ++i) r[i] += y * (aq[i] - theta[col] * q[i]);
        }
        massTimes(r.data(), mw.data());
        const double rn = std::sqrt(std::max(dot(r, mw.data()), 0.0));
        if (!(rn <= 1e-9 * std::fabs(theta[col]))) converged = false;
      }
    }
    if (converged || cols >= mMax) break;
    int added = 0;
    for (auto& v : next)
      if ((int)(Q.size() / n) < mMax && addVector(v)) ++added;
    if (added == 0) {  // the Krylov space is exhausted: the Ritz values are exact
      converged = cols >= nmod;
      break;
    }
  }
  eng.endStiffnessSolves();
  if (rc) return rc;
  const int cols = (int)(AQ.size() / n);
  if (cols < nmod || (int)theta.size() != cols) return -5;
  lambda.assign(nmod, 0.0);
  vecs.assign((size_t)n * nmod, 0.0);
  nNeg = 0;
  for (int k = 0; k < nmod; ++k) {
    const int col = cols - 1 - k;
    lambda[k] = 1.0 / theta[col];
    if (lambda[k] < 0.0) ++nNeg;
    double* v = &vecs[(size_t)n * k];
    for (int s2 = 0; s2 < cols; ++s2) {
      const double c = Y[(size_t)s2 + (size_t)cols * col];
      const double* q = &Q[(size_t)n * s2];
      for (int i = 0; i < n; ++i) v[i] += c * q[i];
    }
  }
  return converged ? 0 : 1;  // 1: not every requested mode reached the tolerance
}

}  // namespace fgpu
