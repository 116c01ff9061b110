// host_model.cpp -- reading a FEDEM solver input (.fsi subset) and the
// solver options, and building the flat model arrays the GPU engine uploads.
//
// Reference behaviour restated here (paths relative to fedem-solvers):
//   namelist records   src/vpmCommon/triadTypeModule.f90:1264, supElTypeModule.f90:1301-1365,
//                      src/vpmSolver/finiteElementModule.f90:151-205, forceTypeModule.f90:157-260
//   options/defaults   src/vpmSolver/solverInterface.C:195-554
//   Newmark constants  src/vpmSolver/initiateSystemTypeModule.f90:74-92
//   beam matrices      src/vpmSolver/finiteElementModule.f90:283-541 -> src/Femlib/beam.f
//                      (BEAM31 :11, BELS31 :619, BEAM35 :396), src/Femlib/beamaux.f
//   offsets/corot init src/vpmSolver/initiateSupElTypeModule.f90:354-371, supElTypeModule.f90:779-992
//   SAM numbering      src/vpmSolver/samSolverModule.f90:95-250 (triads in input order, MSC = BC)
//   damping/scaling    src/vpmSolver/initiateSupElTypeModule.f90:549-599, :740-811
//   reduced parts      src/vpmSolver/initiateSupElTypeModule.f90:140-700, 962-1033 (ReadSupEls,
//                      ReadSupElMatrices), samSolverModule.f90:137-148 (generalized DOFs)

#include "host_model.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <array>
#include <climits>
#include <map>
#include <string_view>

namespace fgpu {
namespace {

// ---------------------------------------------------------------------------
// Namelist text -> records of key -> raw value tokens
// ---------------------------------------------------------------------------
// One namelist record, flat: its keys (lower case) in first-seen order and
// the values of every key occurrence as segments of one value list (a key
// given twice collects both segments, in order).  Values are views of the
// model text as written (quotes of quoted strings removed; n*v repeats
// expanded); the text outlives the records.
struct NmlRecord {
  std::string name;
  std::vector<std::string> keys;
  std::vector<std::array<int, 3>> segs;  // key index, first value, value count
  std::vector<std::string_view> vals;
  int keyIndex(const char* k) const {
    for (size_t i = 0; i < keys.size(); ++i)
      if (keys[i] == k) return (int)i;
    return -1;
  }
  // the values of key k, in order (false: no such key)
  template <typename F>
  bool each(const char* k, F f) const {
    const int ki = keyIndex(k);
    if (ki < 0) return false;
    for (const auto& sg : segs)
      if (sg[0] == ki)
        for (int v = 0; v < sg[2]; ++v) f(vals[sg[1] + v]);
    return true;
  }
  // the first value of key k (false: no such key or no value)
  bool first(const char* k, std::string_view& out) const {
    const int ki = keyIndex(k);
    if (ki < 0) return false;
    for (const auto& sg : segs)
      if (sg[0] == ki && sg[2] > 0) {
        out = vals[sg[1]];
        return true;
      }
    return false;
  }
};

std::string lowerCase(const std::string& s) {
  std::string r(s);
  std::transform(r.begin(), r.end(), r.begin(), [](unsigned char c) { return (char)std::tolower(c); });
  return r;
}

double toDouble(std::string_view tok) {
  // a Fortran exponent letter d/D reads as e
  char buf[64];
  if (tok.size() < sizeof buf) {
    for (size_t k = 0; k < tok.size(); ++k) buf[k] = (tok[k] == 'd' || tok[k] == 'D') ? 'e' : tok[k];
    buf[tok.size()] = '\0';
    return std::strtod(buf, nullptr);
  }
  std::string t(tok);
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(t.c_str(), nullptr);
}

std::vector<NmlRecord> readNamelists(const char* text) {
  std::vector<NmlRecord> out;
  const size_t n = std::strlen(text);
  size_t p = 0;
  auto lowerIn = [](std::string& r) {
    for (char& ch : r)
      if (ch >= 'A' && ch <= 'Z') ch = (char)(ch - 'A' + 'a');
  };
  // ASCII classes (the model text is ASCII; no locale look-ups per character)
  auto isSpace = [](char ch) { return ch == ' ' || ch == '\n' || ch == '\t' || ch == '\r' || ch == '\f' || ch == '\v'; };
  auto isWordChar = [](char ch) {
    return (ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || (ch >= '0' && ch <= '9') || ch == '_';
  };
  while (p < n) {
    {
      const void* amp = std::memchr(text + p, '&', n - p);
      p = amp ? (size_t)((const char*)amp - text) : n;
    }
    if (p >= n) break;
    size_t q = ++p;
    while (q < n && isWordChar(text[q])) ++q;
    NmlRecord rec;
    rec.name.assign(text + p, q - p);
    lowerIn(rec.name);
    p = q;
    // a word followed by '=' starts a key; words and quoted strings after a
    // key are its values; a word is held back until the next token shows
    // which of the two it is
    int key = -1;
    size_t pendS = 0, pendL = 0;
    bool pend = false;
    auto addValue = [&](const char* v, size_t len, bool word) {
      if (key < 0) return;
      const void* star = word ? std::memchr(v, '*', len) : nullptr;
      if (star && star != v) {
        const size_t sp = (size_t)((const char*)star - v);
        const int rep = std::atoi(std::string(v, sp).c_str());
        for (int r = 0; r < rep; ++r) rec.vals.emplace_back(v + sp + 1, len - sp - 1);  // views
        rec.segs.back()[2] += rep > 0 ? rep : 0;
      } else {
        rec.vals.emplace_back(v, len);
        rec.segs.back()[2] += 1;
      }
    };
    auto flushPending = [&]() {
      if (pend) addValue(text + pendS, pendL, true);
      pend = false;
    };
    while (p < n) {
      const char ch = text[p];
      if (ch == '/') { ++p; break; }
      if (isSpace(ch) || ch == ',') { ++p; continue; }
      if (ch == '!') { while (p < n && text[p] != '\n') ++p; continue; }
      if (ch == '=') {
        ++p;
        if (pend) {  // the held word is a key
          std::string k(text + pendS, pendL);
          lowerIn(k);
          int ki = rec.keyIndex(k.c_str());
          if (ki < 0) {
            ki = (int)rec.keys.size();
            rec.keys.push_back(std::move(k));
          }
          key = ki;
          rec.segs.push_back({ki, (int)rec.vals.size(), 0});
          pend = false;
        }
        continue;
      }
      if (ch == '\'' || ch == '"') {
        flushPending();
        const size_t s0 = ++p;
        while (p < n && text[p] != ch) ++p;
        addValue(text + s0, p - s0, false);
        if (p < n) ++p;
        continue;
      }
      flushPending();
      const size_t s0 = p;
      while (p < n && !isSpace(text[p]) && text[p] != ',' && text[p] != '=' &&
             text[p] != '/' && text[p] != '\'' && text[p] != '"')
        ++p;
      pendS = s0;
      pendL = p - s0;
      pend = true;
    }
    flushPending();
    out.push_back(std::move(rec));
  }
  return out;
}

struct Rec {
  const NmlRecord& r;
  std::vector<double> nums(const char* k) const {
    std::vector<double> v;
    r.each(k, [&](std::string_view x) { v.push_back(toDouble(x)); });
    return v;
  }
  double num(const char* k, double def) const {
    std::string_view x;
    return r.first(k, x) ? toDouble(x) : def;
  }
  int inum(const char* k, int def) const { return (int)std::lround(num(k, (double)def)); }
  std::string str(const char* k) const {
    std::string_view x;
    return r.first(k, x) ? lowerCase(std::string(x)) : std::string();
  }
  // every value as written (file names)
  std::vector<std::string> strs(const char* k) const {
    std::vector<std::string> v;
    r.each(k, [&](std::string_view x) { v.emplace_back(x); });
    return v;
  }
  // the value as written (quotes removed), for names compared case-sensitively
  std::string raw(const char* k) const {
    std::string_view x;
    if (!r.first(k, x)) return std::string();
    std::string v(x);
    if (v.size() >= 2 && (v.front() == '\'' || v.front() == '"') && v.back() == v.front()) v = v.substr(1, v.size() - 2);
    return v;
  }
};

// ---------------------------------------------------------------------------
// Options: -name=value, -name, -name-, -name+
// ---------------------------------------------------------------------------
struct Opts {
  std::map<std::string, std::string> kv;
  explicit Opts(int argc, const char* const* argv) {
    for (int a = 0; a < argc; ++a) {
      if (!argv || !argv[a] || argv[a][0] != '-') continue;
      std::string s(argv[a] + 1), key, val = "true";
      size_t eq = s.find('=');
      if (eq != std::string::npos) {
        key = s.substr(0, eq);
        val = s.substr(eq + 1);
        if (val.size() >= 2 && (val[0] == '"' || val[0] == '\'') && val.back() == val[0])
          val = val.substr(1, val.size() - 2);
      } else if (!s.empty() && (s.back() == '-' || s.back() == '+')) {
        val = s.back() == '-' ? "false" : "true";
        key = s.substr(0, s.size() - 1);
      } else {
        key = s;
      }
      kv[lowerCase(key)] = val;
    }
  }
  double d(const char* k, double def) const {
    auto it = kv.find(lowerCase(k));
    return it == kv.end() ? def : toDouble(it->second);
  }
  int i(const char* k, int def) const { return (int)std::lround(d(k, (double)def)); }
  bool b(const char* k, bool def) const {
    auto it = kv.find(lowerCase(k));
    if (it == kv.end()) return def;
    std::string v = lowerCase(it->second);
    return v == "true" || v == "1" || v == "t" || v == "yes" || v == "on";
  }
  std::string s(const char* k) const {
    auto it = kv.find(lowerCase(k));
    return it == kv.end() ? std::string() : it->second;
  }
};

// ---------------------------------------------------------------------------
// Binary matrix files of reduced parts (ReadSupElMatrices,
// initiateSupElTypeModule.f90:962-1033; readDoubleDBfile,
// binaryDBInterface.f90:387-435; binaryDB.c:643-731): the file opens with the
// tag text '#FEDEM <type>', its header ends with the version field ';1.0;\n'
// and the values follow as raw little-endian doubles, column by column, to the
// end of the file.  The bytes between the tag text and the version field (an
// endian mark and checksum in the reference's tag layout) are not read.  A
// relative name is taken relative to the directory of the model file
// (-fsifile), else the working directory.
// ---------------------------------------------------------------------------
int readMatrixFile(const std::string& name, const std::string& fsiFile, const char* type, size_t nval,
                   std::vector<double>& out, std::string& err) {
  std::string path = name;
  if (!path.empty() && path[0] != '/' && !fsiFile.empty()) {
    const size_t slash = fsiFile.find_last_of('/');
    if (slash != std::string::npos) path = fsiFile.substr(0, slash + 1) + path;
  }
  FILE* f = path.empty() ? nullptr : std::fopen(path.c_str(), "rb");
  if (!f) { err = "cannot open the " + std::string(type) + " file '" + path + "'"; return -80; }
  std::vector<char> buf;
  char chunk[65536];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  std::fclose(f);
  const std::string tag = std::string("#FEDEM ") + type, ver = ";1.0;\n";
  const size_t bytes = 8 * nval;
  if (buf.size() < tag.size() + ver.size() + bytes || std::memcmp(buf.data(), tag.data(), tag.size()) != 0 ||
      std::memcmp(buf.data() + buf.size() - bytes - ver.size(), ver.data(), ver.size()) != 0) {
    err = "'" + path + "' is not a " + type + " file of " + std::to_string(nval) + " values";
    return -81;
  }
  out.resize(nval);
  std::memcpy(out.data(), buf.data() + buf.size() - bytes, bytes);
  return 0;
}

// ---------------------------------------------------------------------------
// Small dense helpers. P34 is a 3x4 position matrix, column-major (12 doubles).
// ---------------------------------------------------------------------------
inline double& at34(double* T, int r, int c) { return T[r + 3 * c]; }
inline double at34(const double* T, int r, int c) { return T[r + 3 * c]; }

void compose34(const double* a, const double* b, double* out) {  // a o b
  double r[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = at34(a, i, 0) * at34(b, 0, j) + at34(a, i, 1) * at34(b, 1, j) + at34(a, i, 2) * at34(b, 2, j);
      if (j == 3) s += at34(a, i, 3);
      r[i + 3 * j] = s;
    }
  std::memcpy(out, r, sizeof(r));
}

void inverse34(const double* a, double* out) {
  double r[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r[i + 3 * j] = at34(a, j, i);
  for (int i = 0; i < 3; ++i)
    r[i + 9] = -(r[i] * a[9] + r[i + 3] * a[10] + r[i + 6] * a[11]);
  std::memcpy(out, r, sizeof(r));
}

void crossp(const double* a, const double* b, double* c) {
  double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
  c[0] = x; c[1] = y; c[2] = z;
}

// Frame through three points: x along p1->p2, z normal to the plane, origin p1.
int frameFrom3Points(const double* p1, const double* p2, const double* p3, double* T) {
  double ex[3], v2[3], ez[3], ey[3];
  for (int k = 0; k < 3; ++k) { ex[k] = p2[k] - p1[k]; v2[k] = p3[k] - p1[k]; }
  crossp(ex, v2, ez);
  double lx = ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2];
  if (!(lx > 1.0e-16)) return -1;
  lx = std::sqrt(lx);
  for (double& v : ex) v /= lx;
  double lz = ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2];
  if (!(lz > 1.0e-16)) return -2;
  lz = std::sqrt(lz);
  for (double& v : ez) v /= lz;
  crossp(ez, ex, ey);
  for (int k = 0; k < 3; ++k) { T[k] = ex[k]; T[3 + k] = ey[k]; T[6 + k] = ez[k]; T[9 + k] = p1[k]; }
  return 0;
}

// Rotation tensor (column-major 3x3) from a rotation vector through a unit
// quaternion (rotationModule.f90:355-370, 393-436, 478-500)
void rotvecToMat(const double* rv, double* R) {
  const double epsTh2 = 0.0005;
  const double thh = 0.5 * std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double fac;
  if (thh < epsTh2) {
    const double f1 = thh / epsTh2;
    fac = f1 * std::sin(epsTh2) / epsTh2 + 1.0 - f1;
  } else {
    fac = std::sin(thh) / thh;
  }
  double q[4] = {std::cos(thh), rv[0] * fac * 0.5, rv[1] * fac * 0.5, rv[2] * fac * 0.5};
  for (int pass = 0; pass < 2; ++pass) {
    const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (double& v : q) v /= n;
  }
  R[0] = 2.0 * (q[1] * q[1] + q[0] * q[0]) - 1.0;
  R[4] = 2.0 * (q[2] * q[2] + q[0] * q[0]) - 1.0;
  R[8] = 2.0 * (q[3] * q[3] + q[0] * q[0]) - 1.0;
  R[3] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
  R[6] = 2.0 * (q[1] * q[3] + q[2] * q[0]);
  R[7] = 2.0 * (q[2] * q[3] - q[1] * q[0]);
  R[1] = 2.0 * (q[2] * q[1] + q[3] * q[0]);
  R[2] = 2.0 * (q[3] * q[1] - q[2] * q[0]);
  R[5] = 2.0 * (q[3] * q[2] + q[1] * q[0]);
}

// Re-orthonormalise the rotation part of a 3x4 matrix through its quaternion
// (rotationModule.f90:447-476, 478-500)
void orthonormRot34(double* T) {
  auto r = [&](int i, int j) { return T[i + 3 * j]; };
  double q[4];
  const double tr = r(0, 0) + r(1, 1) + r(2, 2);
  int imax = 0;
  if (r(1, 1) > r(imax, imax)) imax = 1;
  if (r(2, 2) > r(imax, imax)) imax = 2;
  if (tr > r(imax, imax)) {
    q[0] = std::sqrt(1.0 + tr) * 0.5;
    q[1] = (r(2, 1) - r(1, 2)) / (4.0 * q[0]);
    q[2] = (r(0, 2) - r(2, 0)) / (4.0 * q[0]);
    q[3] = (r(1, 0) - r(0, 1)) / (4.0 * q[0]);
  } else {
    const int i = imax, j = (imax + 1) % 3, k = (imax + 2) % 3;
    q[i + 1] = std::sqrt(r(i, i) * 0.5 + (1.0 - tr) * 0.25);
    q[0] = (r(k, j) - r(j, k)) / (4.0 * q[i + 1]);
    q[j + 1] = (r(j, i) + r(i, j)) / (4.0 * q[i + 1]);
    q[k + 1] = (r(k, i) + r(i, k)) / (4.0 * q[i + 1]);
  }
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (double& v : q) v /= n;
  T[0] = 2.0 * (q[1] * q[1] + q[0] * q[0]) - 1.0;
  T[4] = 2.0 * (q[2] * q[2] + q[0] * q[0]) - 1.0;
  T[8] = 2.0 * (q[3] * q[3] + q[0] * q[0]) - 1.0;
  T[3] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
  T[6] = 2.0 * (q[1] * q[3] + q[2] * q[0]);
  T[7] = 2.0 * (q[2] * q[3] - q[1] * q[0]);
  T[1] = 2.0 * (q[2] * q[1] + q[3] * q[0]);
  T[2] = 2.0 * (q[3] * q[1] - q[2] * q[0]);
  T[5] = 2.0 * (q[3] * q[2] + q[1] * q[0]);
}

// ---------------------------------------------------------------------------
// 12-DOF beam element matrices in superelement axes (Femlib BEAM31/BEAM35).
// E is column-major; e(i,j) uses 1-based indices like the element library.
// ---------------------------------------------------------------------------
struct Mat12 {
  double* a;
  double& operator()(int i, int j) const { return a[(i - 1) + 12 * (j - 1)]; }
};

// Rows of G are the local unit axes in superelement coordinates (DCOS30).
void localAxes(const double* X1, const double* X2, const double* X3, double G[3][3]) {
  double d[3] = {X2[0] - X1[0], X2[1] - X1[1], X2[2] - X1[2]};
  double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (int k = 0; k < 3; ++k) G[0][k] = d[k] / l;
  double w[3] = {X3[0] - X1[0], X3[1] - X1[1], X3[2] - X1[2]};
  double y[3] = {G[0][2] * w[1] - G[0][1] * w[2], G[0][0] * w[2] - G[0][2] * w[0], G[0][1] * w[0] - G[0][0] * w[1]};
  l = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  for (int k = 0; k < 3; ++k) G[1][k] = y[k] / l;
  double z[3] = {G[0][1] * G[1][2] - G[0][2] * G[1][1], G[0][2] * G[1][0] - G[0][0] * G[1][2],
                 G[0][0] * G[1][1] - G[0][1] * G[1][0]};
  l = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  for (int k = 0; k < 3; ++k) G[2][k] = z[k] / l;
}

// E := blockdiag(G)^T E blockdiag(G), 3x3 blocks, then symmetrised from the lower part.
void congruence(double* E, const double G[3][3]) {
  Mat12 e{E};
  for (int bi = 0; bi < 12; bi += 3)
    for (int bj = 0; bj < 12; bj += 3) {
      double B[3][3] = {{0.0}};
      for (int ia = 1; ia <= 3; ++ia)
        for (int ka = 1; ka <= 3; ++ka)
          for (int ja = 1; ja <= 3; ++ja) B[ja - 1][ia - 1] += G[ka - 1][ja - 1] * e(bj + ka, bi + ia);
      for (int ia = 1; ia <= 3; ++ia)
        for (int ka = 1; ka <= 3; ++ka) {
          double s = 0.0;
          for (int ja = 1; ja <= 3; ++ja) s += B[ka - 1][ja - 1] * G[ja - 1][ia - 1];
          e(bj + ka, bi + ia) = s;
        }
    }
  for (int i = 1; i <= 12; ++i)
    for (int j = i; j <= 12; ++j) e(i, j) = e(j, i);
}

// Move the element ends to eccentric nodes (TRIX30); zero eccentricity is a no-op
// apart from exact zero additions, kept for bitwise agreement with the library.
void eccentricNodes(double* E, const double* e1, const double* e2) {
  Mat12 a{E};
  for (int i = 1; i <= 12; ++i) {
    a(4, i) += e1[2] * a(2, i) - e1[1] * a(3, i);
    a(5, i) += -e1[2] * a(1, i) + e1[0] * a(3, i);
    a(6, i) += e1[1] * a(1, i) - e1[0] * a(2, i);
    a(10, i) += e2[2] * a(8, i) - e2[1] * a(9, i);
    a(11, i) += -e2[2] * a(7, i) + e2[0] * a(9, i);
    a(12, i) += e2[1] * a(7, i) - e2[0] * a(8, i);
  }
  for (int i = 1; i <= 12; ++i) {
    a(i, 4) += e1[2] * a(i, 2) - e1[1] * a(i, 3);
    a(i, 5) += -e1[2] * a(i, 1) + e1[0] * a(i, 3);
    a(i, 6) += e1[1] * a(i, 1) - e1[0] * a(i, 2);
    a(i, 10) += e2[2] * a(i, 8) - e2[1] * a(i, 9);
    a(i, 11) += -e2[2] * a(i, 7) + e2[0] * a(i, 9);
    a(i, 12) += e2[1] * a(i, 7) - e2[0] * a(i, 8);
  }
}

// Timoshenko beam stiffness, local axes (BELS31): EP = E,G,A,Iy,Iz,It.
void beamStiffnessLocal(double* E, double L, const double* EP, const double* CA, const double* XS) {
  double EA, EIy, EIz, GIt, phiY, phiZ;
  if (EP[0] < -1.0e-16) {  // generic section data: EA, EI, GAs, GIt given directly
    EA = EP[2]; EIy = EP[3]; EIz = EP[4]; GIt = EP[5];
    phiY = CA[0] > 1.0e-16 ? 12.0 * EIy / (CA[0] * L * L) : 0.0;
    phiZ = CA[1] > 1.0e-16 ? 12.0 * EIz / (CA[1] * L * L) : 0.0;
  } else {
    EA = EP[0] * EP[2]; EIy = EP[0] * EP[3]; EIz = EP[0] * EP[4]; GIt = EP[1] * EP[5];
    phiY = 12.0 * CA[0] * EIy / (EP[2] * EP[1] * L * L);
    phiZ = 12.0 * CA[1] * EIz / (EP[2] * EP[1] * L * L);
  }
  std::fill(E, E + 144, 0.0);
  Mat12 k{E};
  k(1, 1) = EA / L;
  k(2, 2) = 12. * EIy / (L * L * L * (1. + phiY));
  k(3, 3) = 12. * EIz / (L * L * L * (1. + phiZ));
  k(4, 4) = GIt / L;
  k(3, 5) = -.5 * L * k(3, 3);
  k(2, 6) = .5 * L * k(2, 2);
  k(5, 5) = EIz * (4. + phiZ) / (L * (1. + phiZ));
  k(6, 6) = EIy * (4. + phiY) / (L * (1. + phiY));
  k(1, 7) = -k(1, 1);
  k(7, 7) = k(1, 1);
  k(2, 8) = -k(2, 2);
  k(6, 8) = -k(2, 6);
  k(8, 8) = k(2, 2);
  k(3, 9) = -k(3, 3);
  k(5, 9) = -k(3, 5);
  k(9, 9) = k(3, 3);
  k(4, 10) = -k(4, 4);
  k(10, 10) = k(4, 4);
  k(3, 11) = k(3, 5);
  k(5, 11) = EIz * (2. - phiZ) / (L * (1. + phiZ));
  k(9, 11) = -k(3, 5);
  k(11, 11) = k(5, 5);
  k(2, 12) = k(2, 6);
  k(6, 12) = EIy * (2. - phiY) / (L * (1. + phiY));
  k(8, 12) = -k(2, 6);
  k(12, 12) = k(6, 6);
  for (int i = 1; i <= 12; ++i)
    for (int j = 1; j < i; ++j) k(i, j) = k(j, i);
  if (.00001 * std::sqrt(EP[2]) < std::fabs(XS[0]) + std::fabs(XS[1])) {  // shear centre offset
    double ys = XS[0], zs = XS[1];
    for (int i = 1; i <= 12; ++i) {
      k(4, i) = k(4, i) - zs * k(2, i) + ys * k(3, i);
      k(10, i) = k(10, i) - zs * k(8, i) + ys * k(9, i);
    }
    for (int i = 1; i <= 12; ++i) {
      k(i, 4) = k(i, 4) - k(i, 2) * zs + k(i, 3) * ys;
      k(i, 10) = k(i, 10) - k(i, 8) * zs + k(i, 9) * ys;
    }
  }
}

// Consistent mass, local axes (BEAM35, IOP = 3).
void beamMassLocal(double* E, double L, double A, double rho, double Ix) {
  std::fill(E, E + 144, 0.0);
  Mat12 m{E};
  double am = L * A * rho, am2 = L * am, am3 = L * am2, rm = Ix * rho;
  m(1, 1) = am / 3.;
  m(1, 7) = am / 6.;
  m(2, 2) = 13. * am / 35.;
  m(2, 6) = 11. * am2 / 210.;
  m(2, 8) = 9. * am / 70.;
  m(2, 12) = -13. * am2 / 420.;
  m(3, 3) = m(2, 2);
  m(3, 5) = -m(2, 6);
  m(3, 9) = m(2, 8);
  m(3, 11) = -m(2, 12);
  m(4, 4) = L * rm / 3.;
  m(4, 10) = L * rm / 6.;
  m(5, 5) = am3 / 105.;
  m(5, 9) = m(2, 12);
  m(5, 11) = -am3 / 140.;
  m(6, 6) = m(5, 5);
  m(6, 8) = m(3, 11);
  m(6, 12) = m(5, 11);
  m(7, 7) = m(1, 1);
  m(8, 8) = m(2, 2);
  m(8, 12) = m(3, 5);
  m(9, 9) = m(8, 8);
  m(9, 11) = m(2, 6);
  m(10, 10) = m(4, 4);
  m(11, 11) = m(5, 5);
  m(12, 12) = m(6, 6);
  for (int i = 1; i <= 12; ++i)
    for (int j = i; j <= 12; ++j) m(j, i) = m(i, j);
}

struct Prop { int id; double geo[8]; double mat[4]; double zvec[3]; };

int beamMatrices(const Prop& p, const double* und1, const double* und2, double* K, double* M, double* fg,
                 std::string& err) {
  // node positions in superelement axes; no eccentricity (ends at the nodes)
  double X1[3] = {und1[9], und1[10], und1[11]}, X2[3] = {und2[9], und2[10], und2[11]}, X3[3];
  bool hasZ = std::fabs(p.zvec[0]) > 1e-16 || std::fabs(p.zvec[1]) > 1e-16 || std::fabs(p.zvec[2]) > 1e-16;
  if (hasZ) {
    for (int k = 0; k < 3; ++k) X3[k] = X1[k] + p.zvec[k];
  } else {
    // local Z from the default orientation of the beam axis (trans1V)
    double v[3] = {X2[0] - X1[0], X2[1] - X1[1], X2[2] - X1[2]};
    double s2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (!(std::fabs(s2) > 1e-16)) { err = "degenerated beam element (zero length)"; return -1; }
    double s = std::sqrt(s2), t1[3] = {v[0] / s, v[1] / s, v[2] / s}, t2[3], t3[3];
    if (std::fabs(t1[2]) > std::fabs(t1[1])) {
      t2[0] = -t1[1] * t1[0]; t2[1] = t1[0] * t1[0] + t1[2] * t1[2]; t2[2] = -t1[1] * t1[2];
      double l = std::sqrt(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
      for (double& q : t2) q /= l;
      crossp(t1, t2, t3);
    } else {
      t3[0] = -t1[2] * t1[0]; t3[1] = -t1[2] * t1[1]; t3[2] = t1[0] * t1[0] + t1[1] * t1[1];
      double l = std::sqrt(t3[0] * t3[0] + t3[1] * t3[1] + t3[2] * t3[2]);
      for (double& q : t3) q /= l;
    }
    for (int k = 0; k < 3; ++k) X3[k] = X1[k] + t3[k];
  }
  double dx = X2[0] - X1[0], dy = X2[1] - X1[1], dz = X2[2] - X1[2];
  double L = std::sqrt(dx * dx + dy * dy + dz * dz);
  double tolL = 1.0e-6 * (std::fabs(X1[0]) + std::fabs(X2[0]) + std::fabs(X1[1]) + std::fabs(X2[1]) +
                          std::fabs(X1[2]) + std::fabs(X2[2]));
  if (L - tolL <= 0.0) { err = "degenerated beam element"; return -1; }
  double EP[6] = {p.mat[1], p.mat[2], p.geo[0], p.geo[1], p.geo[2], p.geo[3]};
  double CA[2] = {p.geo[4], p.geo[5]}, XS[2] = {p.geo[6], p.geo[7]};
  if (EP[1] <= 1.0e-16 || EP[2] <= 1.0e-16) { err = "invalid beam property parameters"; return -3; }
  double G[3][3];
  localAxes(X1, X2, X3, G);
  const double zero[3] = {0.0, 0.0, 0.0};
  beamStiffnessLocal(K, L, EP, CA, XS);
  congruence(K, G);
  eccentricNodes(K, zero, zero);
  double rho = p.mat[0], Ix = p.geo[1] + p.geo[2];
  if (Ix <= 0.0) Ix = p.geo[3];
  double area = EP[2], rix = Ix;
  if (EP[0] <= 1.0e-16 && rho > 1.0e-16) { area = 1.0; rix = Ix / rho; }
  beamMassLocal(M, L, area, rho, rix);
  congruence(M, G);
  eccentricNodes(M, zero, zero);
  for (int i = 0; i < 12; ++i)
    for (int c = 0; c < 3; ++c) fg[i + 12 * c] = M[i + 12 * c] + M[i + 12 * (c + 6)];
  return 0;
}

void setTol(const Opts& o, const char* key, Control& c, int idx) {
  double v = o.d(key, 0.0);
  c.tolCode[idx] = v > 0.0 ? 1 : v < 0.0 ? 2 : 0;
  c.tolVal[idx] = std::fabs(v);
}

}  // namespace

int buildModel(const char* fsi, int argc, const char* const* argv, HostModel& m, std::string& err) {
  if (!fsi) { err = "no model text"; return -1; }
  Opts o(argc, argv);
  Control& c = m.ctl;
  double a = o.d("alphaNewmark", 0.1);
  a = std::min(std::max(a, 0.0), 1.0 / 3.0);
  c.alpha = -a;
  c.beta = (1.0 - c.alpha) * (1.0 - c.alpha) / 4.0;
  c.gamma = 0.5 - c.alpha;
  c.tStart = o.d("timeStart", 0.0);
  c.tEnd = o.d("timeEnd", 0.0);
  c.tInc = std::max(o.d("timeInc", 0.0), 1.0e-6);
  c.minInc = o.d("minInc", 0.001);
  // initiateSystemTypeModule.f90:98, 125-126 (fixed step size)
  c.maxInc = o.d("maxInc", 0.1);
  if (c.tInc > 0.8 * c.maxInc) c.maxInc = 1.25 * c.tInc;
  c.maxIt = o.i("maxit", 15);
  c.minIt = o.i("minit", 1);
  c.fixedIt = o.i("numit", 0);
  c.nUpdat = o.i("nupdat", 0);
  c.maxSeqNoUpdate = o.i("maxSeqNoUpdate", 100);
  c.stiffDampFiltering = o.i("stiffDampFiltering", 1);
  c.initEquilibrium = o.b("initEquilibrium", false);
  c.tolInitEquil = o.d("tolInitEquil", 1.0e-3);
  c.limInitEquilStep = o.d("limInitEquilStep", 1.0);
  c.tolFactorize = o.d("tolFactorize", 1.0e-12);
  c.tQStatic = o.d("quasiStatic", 0.0);
  if (c.tQStatic <= c.tStart) c.tQStatic = -1.0e99;  // initiateSystemTypeModule.f90:129-132
  const char* tolKeys[18] = {"tolDispNorm", "tolDispTra", "tolDispRot", "tolDispGen", "tolVelNorm", "tolVelTra",
                             "tolVelRot",   "tolVelGen",  "tolAccNorm", "tolAccTra",  "tolAccRot",  "tolAccGen",
                             "tolResNorm",  "tolResTra",  "tolResRot",  "tolResGen",  "tolEnerMax", "tolEnerSum"};
  for (int k = 0; k < 18; ++k) setTol(o, tolKeys[k], c, k);
  // options that change the results and that this path does not implement are
  // refused, never ignored: iteration cut-back (newmarkRoutinesModule.f90:879-896,
  // 979-1009, 1106-1116, active when cutbackFactor < 1), line search (:915-918),
  // geometric stiffness, centripetal force correction, the Newmark variants of
  // NewmarkFlag and tangent updates by tolerance (:826-842, tolUpdateFactor > 1)
  if (o.d("cutbackFactor", 1.0) < 1.0) { err = "iteration cut-back (-cutbackFactor < 1) is not supported"; return -60; }
  if (o.b("cutbackSing", false)) { err = "cut-back on singularities (-cutbackSing) is not supported"; return -60; }
  for (const char* key : {"lineSearch", "stressStiffDyn", "stressStiffEqu", "centripForceCorr"})
    if (o.b(key, false)) { err = std::string("-") + key + " is not supported by the GPU solver"; return -61; }
  if (o.i("NewmarkFlag", 0) != 0) { err = "-NewmarkFlag other than 0 is not supported"; return -62; }
  if (o.d("tolUpdateFactor", 0.0) > 1.0) { err = "tangent updates by tolerance (-tolUpdateFactor > 1) are not supported"; return -63; }

  std::vector<NmlRecord> recs = readNamelists(fsi);
  // record types this path does not implement are refused, never dropped
  for (const NmlRecord& nr : recs)
    for (const char* bad : {"higher_pair", "mass", "user_el", "tire", "road", "supel_load",
                            "spring_yield", "spring_failure", "master_curve", "friction_set", "bushing_element",
                            "contact_element", "damper_base", "external_control_system", "control_variable",
                            "control_line", "control_input", "control_element", "wind_point", "turbine_config",
                            "master_pos", "generic_part"})
      if (nr.name == bad) {
        err = "&" + nr.name + " records are not supported by the GPU solver";
        return -50;
      }
  std::vector<Prop> props;
  std::map<int, int> triIndex;
  // pass 1: mechanism, environment, triads, properties
  for (const NmlRecord& nr : recs) {
    Rec r{nr};
    if (nr.name == "mechanism") {
      c.wDisp[0] = r.num("weighttranslation", 1.0);
      c.wDisp[1] = r.num("weightrotation", 1.0);
      c.wDisp[2] = r.num("weightgeneralized", 1.0);
    } else if (nr.name == "environment") {
      auto g = r.nums("gravity");
      for (size_t k = 0; k < 3 && k < g.size(); ++k) c.gravity[k] = g[k];
    } else if (nr.name == "triad") {
      int id = r.inum("id", 0);
      triIndex[id] = m.ntri++;
      m.triId.push_back(id);
      m.triNdof.push_back(r.inum("ndofs", 6));
      auto u = r.nums("ur");  // 3x4, row by row in the file
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 3; ++row) {
          size_t k = (size_t)(4 * row + col);
          m.ur.push_back(k < u.size() ? u[k] : 0.0);
        }
      auto bc = r.nums("bc");
      for (int k = 0; k < 6; ++k) m.dofType.push_back(k < (int)bc.size() ? (int)std::lround(bc[k]) : 1);
    } else if (nr.name == "element_property") {
      Prop p{};
      p.id = r.inum("id", 0);
      auto g = r.nums("geometry");
      for (size_t k = 0; k < 8 && k < g.size(); ++k) p.geo[k] = g[k];
      auto mt = r.nums("material");
      for (size_t k = 0; k < 4 && k < mt.size(); ++k) p.mat[k] = mt[k];
      auto z = r.nums("orientation");
      for (size_t k = 0; k < 3 && k < z.size(); ++k) p.zvec[k] = z[k];
      props.push_back(p);
    }
  }
  // engines (engineRoutinesModule.f90 subset): value = f(x), x = time for a TIME
  // sensor (or no sensor), else 0; f = SCALE (realData(1) * x), CONSTANT
  // (realData(1)), none (x), or an external function: DEVICE_FUNCTION without
  // a file, whose value on channel `channel` the caller sets (setExtFunc).
  // Stored as x-coefficient eA, constant eB and external channel (0-based, -1 none).
  // SINUSOIDAL: realData = frequency (Hz), delay (periods), amplitude, mean;
  // value mean + amplitude * sin(2 pi (frequency x - delay)) (the first three
  // as the reference's regular-wave use of the function reads them,
  // hydroDynamicsModule.f90:345-349)
  struct FuncDef {
    std::string type;
    double c = 0.0;
    int channel = 0;
    double sine[4] = {0, 0, 0, 0};
  };
  std::map<int, FuncDef> funcs;  // id -> definition
  std::map<int, bool> timeSensor;  // id -> TIME sensor
  for (const NmlRecord& nr : recs) {
    Rec r{nr};
    if (nr.name == "function") {
      auto rd = r.nums("realdata");
      FuncDef fd;
      fd.type = r.str("type");
      fd.c = rd.empty() ? (fd.type == "scale" ? 1.0 : 0.0) : rd[0];
      if (fd.type == "sinusoidal")
        for (size_t k = 0; k < 4 && k < rd.size(); ++k) fd.sine[k] = rd[k];
      if (fd.type == "device_function") {
        if (!r.raw("filename").empty()) { err = "device functions reading a file are not supported"; return -22; }
        fd.channel = r.inum("channel", 0);
        if (fd.channel < 1) { err = "external function without a channel (>= 1)"; return -22; }
      }
      funcs[r.inum("id", 0)] = fd;
    } else if (nr.name == "sensor") {
      timeSensor[r.inum("id", 0)] = r.str("type") == "time";
    }
  }
  struct EngineVal {
    double eA, eB;
    int ch;
    double sine[4];
  };
  std::map<int, EngineVal> engines;  // id -> value coefficients
  for (const NmlRecord& nr : recs) {
    if (nr.name != "engine") continue;
    Rec r{nr};
    int fid = r.inum("functionid", 0), sid = r.inum("argsensorid", 0);
    double xs = 1.0;
    if (sid > 0) {
      auto it = timeSensor.find(sid);
      xs = (it != timeSensor.end() && it->second) ? 1.0 : 0.0;
    }
    double eA = xs, eB = 0.0;
    int ch = -1, ftype = 0;
    double fc = 0.0, sine[4] = {0, 0, 0, 0};
    if (fid > 0) {
      auto it = funcs.find(fid);
      if (it == funcs.end()) { err = "engine refers to unknown function"; return -21; }
      fc = it->second.c;
      if (it->second.type == "scale") { eA = it->second.c * xs; ftype = 1; }
      else if (it->second.type == "constant") { eA = 0.0; eB = it->second.c; ftype = 2; }
      else if (it->second.type == "device_function") { eA = 0.0; ch = it->second.channel - 1; ftype = 3; }
      else if (it->second.type == "sinusoidal") {
        eA = 0.0;
        ftype = 4;
        for (int k = 0; k < 4; ++k) sine[k] = it->second.sine[k];
        sine[0] *= xs;  // frequency 0 without a TIME sensor: a constant
      } else {
        err = "function type '" + it->second.type + "' is not supported (SCALE, CONSTANT, SINUSOIDAL, DEVICE_FUNCTION)";
        return -22;
      }
    }
    const int id = r.inum("id", 0);
    engines[id] = {eA, eB, ch, {sine[0], sine[1], sine[2], sine[3]}};
    for (double v : sine) m.engSin.push_back(v);
    // the engine table for evalFunc / getFuncId (solverModule.f90:1602-1680)
    auto ext = r.nums("extid");
    m.engId.push_back(id);
    m.engUserId.push_back(ext.empty() ? id : (int)std::lround(ext[0]));
    m.engTag.push_back(r.raw("tag"));
    m.engEA.push_back(eA);
    m.engEB.push_back(eB);
    m.engCh.push_back(ch);
    m.engFType.push_back(ftype);
    m.engFc.push_back(fc);
    m.engTimeArg.push_back(xs != 0.0 ? 1 : 0);
    if (ch + 1 > m.nExt) m.nExt = ch + 1;
  }
  // prescribed deflections: MEQN = -ICEQ of the constraint equation (samSolverModule.f90)
  std::vector<int> motionOfDof(6 * (size_t)m.ntri, -1);
  for (const NmlRecord& nr : recs) {
    if (nr.name != "motion") continue;
    Rec r{nr};
    auto it = triIndex.find(r.inum("triadid", 0));
    if (it == triIndex.end()) { err = "motion on unknown triad"; return -23; }
    int dof = r.inum("ldof", 0);
    if (dof < 1 || dof > m.triNdof[it->second]) { err = "motion DOF must be 1..nDOFs of its triad"; return -24; }
    std::string type = r.str("type");
    if (!type.empty() && type != "deflection") { err = "only prescribed deflections are supported"; return -25; }
    int& slot = motionOfDof[6 * (size_t)it->second + dof - 1];
    if (slot >= 0) { err = "two motions on one DOF"; return -26; }
    slot = (int)m.motD0.size();
    double eA = 0.0, eB = 0.0, d1 = r.num("d1", 0.0);
    int ch = -1;
    int eid = r.inum("motionengineid", 0);
    if (eid > 0) {
      auto e = engines.find(eid);
      if (e == engines.end()) { err = "motion refers to unknown engine"; return -27; }
      eA = e->second.eA;
      eB = e->second.eB;
      ch = e->second.ch;
      if (e->second.sine[2] != 0.0 || e->second.sine[3] != 0.0) {
        err = "prescribed motions driven by a SINUSOIDAL function are not supported";
        return -27;
      }
    } else {
      d1 = 0.0;
    }
    m.motD0.push_back(r.num("d0", 0.0));
    m.motD1.push_back(d1);
    m.motEA.push_back(eA);
    m.motEB.push_back(eB);
    m.motCh.push_back(ch);
    if (c.initEquilibrium && m.motD0.back() + d1 * (eA * c.tStart + eB) != 0.0) {
      err = "prescribed start values other than zero with initEquilibrium are not supported";
      return -28;
    }
  }
  // master-slave joints (initiateJointTypeModule.f90:120-600): one master
  // triad; joint variables JointVarDefs = (lDof, iMat) pairs with at most one
  // rotation per position matrix; no joint springs, dampers or friction
  struct JointIn {
    int slave, master, nMats = 0;
    std::vector<int> ldof, imat, bc;
    std::vector<double> v0;
    double PJG[12];
  };
  std::vector<JointIn> jin;
  for (const NmlRecord& nr : recs) {
    if (nr.name != "masterslavejoint") continue;
    Rec r{nr};
    const int type = r.inum("type", 0);
    if (type != 1 && type != 3 && type != 4) {
      err = "only point-to-point revolute, rigid and free joints (type 1, 3, 4) are supported";
      return -70;
    }
    if (r.inum("version", 0) < 0) { err = "free joints without rotation coupling are not supported"; return -70; }
    JointIn J;
    auto si = triIndex.find(r.inum("slaveid", 0)), mi = triIndex.find(r.inum("masterid", 0));
    if (si == triIndex.end() || mi == triIndex.end() || si->second == mi->second) {
      err = "joint with an invalid dependent or independent triad";
      return -71;
    }
    J.slave = si->second;
    J.master = mi->second;
    if (m.triNdof[J.slave] != 6) { err = "the dependent triad of a joint needs 6 DOFs"; return -72; }
    for (const char* key : {"springid", "damperid", "frictionsetid", "frictionspringid", "frictionengineid"})
      for (double v : r.nums(key))
        if (v > 0.0) { err = "joint springs, dampers and friction are not supported"; return -73; }
    const int nv = r.inum("njointvars", 0);
    auto defs = r.nums("jointvardefs"), bc = r.nums("bc"), v0 = r.nums("jvarinitval");
    for (int k = 0; k < nv; ++k) {
      const int ld = 2 * k < (int)defs.size() ? (int)std::lround(defs[2 * k]) : 0;
      const int im = 2 * k + 1 < (int)defs.size() ? (int)std::lround(defs[2 * k + 1]) : 0;
      if (ld < 1 || ld > 6 || im < 1) { err = "invalid joint variable definition"; return -74; }
      J.ldof.push_back(ld);
      J.imat.push_back(im);
      J.bc.push_back(k < (int)bc.size() ? (int)std::lround(bc[k]) : 1);
      J.v0.push_back(k < (int)v0.size() ? v0[k] : 0.0);
      J.nMats = std::max(J.nMats, im);
    }
    for (int im = 1; im <= J.nMats; ++im) {
      int nrot = 0;
      for (int k = 0; k < nv; ++k) nrot += J.imat[k] == im && J.ldof[k] > 3;
      if (nrot > 1) { err = "joints with several rotations in one position matrix are not supported"; return -75; }
    }
    auto pg = r.nums("initposinglobal");  // 3x4 row by row
    for (int col = 0; col < 4; ++col)
      for (int row = 0; row < 3; ++row) {
        const size_t k = (size_t)(4 * row + col);
        J.PJG[row + 3 * col] = k < pg.size() ? pg[k] : 0.0;
      }
    orthonormRot34(J.PJG);
    jin.push_back(J);
  }
  for (size_t a = 0; a < jin.size(); ++a)
    for (size_t b = 0; b < jin.size(); ++b)
      if (a != b && (jin[a].slave == jin[b].slave || jin[a].master == jin[b].slave)) {
        err = "a triad dependent in two joints, or chained joints, are not supported";
        return -76;
      }
  if (!jin.empty() && !m.motD0.empty()) { err = "joints together with prescribed motions are not supported"; return -77; }
  if (!jin.empty() && c.tQStatic > c.tStart && c.fixedIt == -1) {
    err = "joints together with pure linear quasi-static steps are not supported";
    return -77;
  }
  if (!m.motD0.empty() && c.tQStatic > c.tStart && c.fixedIt < -1) {
    err = "quasi-static steps need numit = -1 (linear) or numit >= 0";
    return -29;
  }
  for (double w = 0; w < 3; ++w) {
    int k = (int)w;
    c.wForce[k] = c.wDisp[k] > 0.0 ? 1.0 / c.wDisp[k] : 0.0;
  }
  // SAM: DOFs per triad in input order; status code BC: 0 fixed, 1 free,
  // 2 free except in the initial equilibrium iterations
  // (initiateTriadTypeModule.f90:57-123)
  std::vector<int> bcs = m.dofType;  // temporarily holds the BC codes, 6 per triad
  m.dofType.clear();
  m.triFirstDof.resize(m.ntri);
  std::vector<int> slaveOf(m.ntri, -1);
  for (size_t j = 0; j < jin.size(); ++j) slaveOf[jin[j].slave] = (int)j;
  for (int t = 0; t < m.ntri; ++t) {
    m.triFirstDof[t] = m.ndof;
    for (int k = 0; k < m.triNdof[t]; ++k) {
      int bc = bcs[6 * t + k];
      if (slaveOf[t] >= 0) {  // dependent DOF of a joint: no equation (samSolverModule.f90:613-633)
        if (bc != 1 && !(bc == 2 && !c.initEquilibrium)) { err = "a joint's dependent triad must be free"; return -78; }
        m.meqn.push_back(-1);
        m.dofType.push_back(k < 3 ? 1 : 2);
        continue;
      }
      if (bc == 2 && !c.initEquilibrium) bc = 1;
      if (bc != 0 && bc != 1) { err = "BC code other than 0, 1 or 2 (2 only without initEquilibrium)"; return -30; }
      const int mot = motionOfDof[6 * (size_t)t + k];
      if (mot >= 0) {
        m.meqn.push_back(-2 - mot);
        m.motDof.push_back(m.ndof + k);
      } else {
        m.meqn.push_back(bc == 1 ? m.neq++ : -1);
      }
      m.dofType.push_back(k < 3 ? 1 : 2);
    }
    m.ndof += m.triNdof[t];
  }
  m.dofDep.assign(m.ndof, -1);
  for (size_t j = 0; j < jin.size(); ++j)
    for (int k = 0; k < 6; ++k) m.dofDep[m.triFirstDof[jin[j].slave] + k] = 6 * (int)j + k;
  // generalized DOFs of the reduced parts after the triad DOFs, part by part
  // (initSAM_dofStatus, samSolverModule.f90:137-148, 191-197); status codes
  // from the part's BC list (default free)
  auto isPart = [](const Rec& r) {
    auto f = r.strs("inputfiles");
    return !f.empty() && !f[0].empty();
  };
  for (const NmlRecord& nr : recs) {
    if (nr.name != "sup_el") continue;
    Rec r{nr};
    if (!isPart(r)) continue;
    const int ng = r.inum("numgendofs", 0);
    if (ng < 0) { err = "negative numGenDOFs"; return -10; }
    auto bcg = r.nums("bc");
    m.pGenFirstDof.push_back(m.ndof);
    for (int g = 0; g < ng; ++g) {
      int bc = g < (int)bcg.size() ? (int)std::lround(bcg[g]) : 1;
      if (bc == 2 && !c.initEquilibrium) bc = 1;
      if (bc != 0 && bc != 1) { err = "generalized DOF BC other than 0, 1 or 2"; return -30; }
      m.meqn.push_back(bc == 1 ? m.neq++ : -1);
      m.dofType.push_back(3);
      m.dofDep.push_back(-1);
    }
    m.ndof += ng;
  }
  // joint DOFs after all triad DOFs (initSAM_dofStatus, samSolverModule.f90:95-250)
  m.njoint = (int)jin.size();
  for (size_t j = 0; j < jin.size(); ++j) {
    const JointIn& J = jin[j];
    const int nv = (int)J.ldof.size();
    m.jSlave.push_back(J.slave);
    m.jMaster.push_back(J.master);
    m.jNM.push_back(std::min(6, m.triNdof[J.master]));
    m.jFirstDof.push_back(m.ndof);
    m.jNdof.push_back(nv);
    m.jNmats.push_back(J.nMats);
    m.jDofOff.push_back((int)m.jLdof.size());
    for (int k = 0; k < nv; ++k) {
      const int bc = J.bc[k];
      if (bc != 0 && bc != 1 && !(bc == 2 && !c.initEquilibrium)) { err = "joint DOF BC other than 0, 1"; return -30; }
      m.meqn.push_back(bc != 0 ? m.neq++ : -1);
      m.dofType.push_back(J.ldof[k] <= 3 ? 1 : 2);
      m.dofDep.push_back(-1);
      m.jLdof.push_back(J.ldof[k]);
      m.jImat.push_back(J.imat[k]);
      m.jVar0.push_back(J.v0[k]);
    }
    m.ndof += nv;
    // joint frame in the master triad's axes and the slave's start position in
    // the joint frame with every joint variable at zero (initiateJointTypeModule.f90:564-598)
    double inv[12], S0[12], tmp[12];
    inverse34(J.PJG, inv);
    compose34(inv, &m.ur[12 * (size_t)J.slave], S0);
    for (int im = J.nMats; im >= 1; --im) {
      double F[12] = {0}, th[3] = {0, 0, 0}, Fi[12];
      for (int k = 0; k < nv; ++k)
        if (J.imat[k] == im) {
          if (J.ldof[k] <= 3) F[9 + J.ldof[k] - 1] = J.v0[k];
          else th[J.ldof[k] - 4] = J.v0[k];
        }
      rotvecToMat(th, F);
      inverse34(F, Fi);
      compose34(Fi, S0, tmp);
      std::memcpy(S0, tmp, sizeof(S0));
    }
    for (double v : S0) m.jSTPos0.push_back(v);
    inverse34(&m.ur[12 * (size_t)J.master], inv);
    compose34(inv, J.PJG, tmp);
    for (double v : tmp) m.jPosInT.push_back(v);
  }
  m.jDofOff.push_back((int)m.jLdof.size());
  for (int j = 0; j < m.njoint; ++j) {
    for (int col = 0; col < 12; ++col) {
      int e = -1;
      if (col < m.jNM[j]) e = m.meqn[m.triFirstDof[m.jMaster[j]] + col];
      else if (col - m.jNM[j] < m.jNdof[j]) e = m.meqn[m.jFirstDof[j] + col - m.jNM[j]];
      if (e < -1) { err = "a joint's independent triad has a prescribed DOF"; return -77; }
      m.jColEq.push_back(e);
    }
  }
  // pass 2: superelements, undeformed positions, loads
  std::map<int, std::vector<std::array<double, 9>>> engineLoads;  // equation -> (f0, f1, eA, eB, channel, sine x4)
  std::vector<int> elProp;
  std::map<int, int> elIndex;
  m.qext.assign(m.neq, 0.0);
  std::map<int, int> partIndex;
  std::vector<std::array<std::string, 3>> partFiles;
  std::vector<std::array<double, 4>> partScale;  // stiffScale, massScale, alpha1, alpha2
  std::vector<std::vector<double>> partA3, partA4;
  for (const NmlRecord& nr : recs) {
    Rec r{nr};
    if (nr.name == "sup_el" && isPart(r)) {
      // a reduced part (SUP_EL with inputFiles; ReadSupEls, initiateSupElTypeModule.f90:140-700)
      const int p = m.npart++;
      partIndex[r.inum("id", 0)] = p;
      const int nt = r.inum("numtriads", 0), ng = r.inum("numgendofs", 0);
      auto tids = r.nums("triadids");
      if (nt < 2 || (int)tids.size() < nt) { err = "a part needs at least two triads"; return -10; }
      // not on this path: nonlinear parts, part load cases, stress stiffening,
      // mass-matrix correction, the shadowPosAlg 2 frame, time-dependent scaling
      if (r.inum("numstates", 0) > 0 || r.inum("numloadcase", 0) > 0) {
        err = "nonlinear parts and part load cases are not supported";
        return -10;
      }
      for (double v : r.nums("stressstiffflag"))
        if (v > 0.0) { err = "stress stiffening of parts is not supported"; return -10; }
      if (r.inum("masscorrflag", -1) > 0) { err = "mass-matrix correction of parts is not supported"; return -10; }
      if (r.inum("shadowposalg", 0) > 1) { err = "only the triangle frame (shadowPosAlg 1) is supported"; return -10; }
      if (r.inum("stiffengineid", 0) > 0 || r.inum("strdmpengineid", 0) > 0) {
        err = "time-dependent part stiffness or damping scaling is not supported";
        return -10;
      }
      m.pNtri.push_back(nt);
      m.pNgen.push_back(ng);
      m.pTriOff.push_back((int)m.pTri.size());
      for (int k = 0; k < nt; ++k) {
        auto it = triIndex.find((int)std::lround(tids[k]));
        if (it == triIndex.end()) { err = "part refers to unknown triad"; return -11; }
        if (m.triNdof[it->second] != 6) { err = "part triads need 6 DOFs"; return -12; }
        m.pTri.push_back(it->second);
      }
      auto sp = r.nums("suppos");
      double S[12];
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 3; ++row) {
          size_t k = (size_t)(4 * row + col);
          S[row + 3 * col] = k < sp.size() ? sp[k] : 0.0;
        }
      const char* refKey[3] = {"reftriad1id", "reftriad2id", "reftriad3id"};
      const char* offKey[3] = {"offset1", "offset2", "offset3"};
      for (int j = 0; j < 3; ++j) {
        int rid = r.inum(refKey[j], 0), node = -1;
        for (int k = 0; k < nt; ++k)
          if (m.triId[m.pTri[m.pTriOff[p] + k]] == rid) node = k;
        if (node < 0) { err = "invalid reference triad"; return -13; }
        m.pRef.push_back(node);
        // offset in the reference triad's axes (TransformOffset, supElTypeModule.f90:779-789)
        auto ov = r.nums(offKey[j]);
        double off[3] = {0, 0, 0}, so[3];
        for (size_t k = 0; k < 3 && k < ov.size(); ++k) off[k] = ov[k];
        for (int q = 0; q < 3; ++q) so[q] = S[q] * off[0] + S[q + 3] * off[1] + S[q + 6] * off[2];
        const double* U = &m.ur[12 * (size_t)m.pTri[m.pTriOff[p] + node]];
        for (int col = 0; col < 3; ++col)
          m.pOffset.push_back(so[0] * U[3 * col] + so[1] * U[3 * col + 1] + so[2] * U[3 * col + 2]);
      }
      for (double v : S) m.pSupTr.push_back(v);
      m.pTrUnd.resize(12 * m.pTri.size(), 0.0);
      auto files = r.strs("inputfiles");
      std::array<std::string, 3> fl;
      for (int k = 0; k < 3; ++k) fl[k] = k < (int)files.size() ? files[k] : std::string();
      partFiles.push_back(fl);
      partScale.push_back({r.num("stiffscale", 1.0), r.num("massscale", 1.0), r.num("alpha1", 0.0),
                           r.num("alpha2", 0.0)});
      auto a3 = r.nums("alpha3"), a4 = r.nums("alpha4");
      a3.resize(ng, 0.0);
      a4.resize(ng, 0.0);
      partA3.push_back(a3);
      partA4.push_back(a4);
    } else if (nr.name == "triad_undpos" && partIndex.count(r.inum("supelid", 0))) {
      const int p = partIndex[r.inum("supelid", 0)], tid = r.inum("triadid", 0);
      int node = -1;
      for (int k = 0; k < m.pNtri[p]; ++k)
        if (m.triId[m.pTri[m.pTriOff[p] + k]] == tid) node = k;
      if (node < 0) { err = "undeformed position for a triad not on the part"; return -16; }
      for (const char* key : {"eccvec", "eccmass"})
        for (double v : r.nums(key))
          if (std::fabs(v) > 1.0e-16) { err = "eccentricity vectors of part triads are not supported"; return -16; }
      auto u = r.nums("undposinsupelsystem");
      double* T = &m.pTrUnd[12 * (size_t)(m.pTriOff[p] + node)];
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 3; ++row) {
          size_t k = (size_t)(4 * row + col);
          T[row + 3 * col] = k < u.size() ? u[k] : 0.0;
        }
    } else if (nr.name == "sup_el") {
      auto tids = r.nums("triadids");
      if (r.inum("numtriads", 2) != 2 || tids.size() < 2) { err = "only 2-noded beam superelements"; return -10; }
      int e = m.nel++;
      elIndex[r.inum("id", 0)] = e;
      m.elId.push_back(r.inum("id", 0));
      int tri[2];
      for (int k = 0; k < 2; ++k) {
        auto it = triIndex.find((int)std::lround(tids[k]));
        if (it == triIndex.end()) { err = "superelement refers to unknown triad"; return -11; }
        tri[k] = it->second;
        if (m.triNdof[tri[k]] != 6) { err = "beam triads need 6 DOFs"; return -12; }
        m.elTri.push_back(tri[k]);
      }
      const char* refKey[3] = {"reftriad1id", "reftriad2id", "reftriad3id"};
      const char* offKey[3] = {"offset1", "offset2", "offset3"};
      auto sp = r.nums("suppos");
      double S[12];
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 3; ++row) {
          size_t k = (size_t)(4 * row + col);
          S[row + 3 * col] = k < sp.size() ? sp[k] : 0.0;
        }
      for (int j = 0; j < 3; ++j) {
        int rid = r.inum(refKey[j], 0), node = -1;
        for (int k = 0; k < 2; ++k)
          if (m.triId[tri[k]] == rid) node = k;
        if (node < 0) { err = "invalid reference triad"; return -13; }
        m.elRef.push_back(node);
        // offset expressed in the reference triad axes: ur^T * (supPos * offset)
        auto ov = r.nums(offKey[j]);
        double off[3] = {0, 0, 0}, so[3];
        for (size_t k = 0; k < 3 && k < ov.size(); ++k) off[k] = ov[k];
        for (int q = 0; q < 3; ++q) so[q] = S[q] * off[0] + S[q + 3] * off[1] + S[q + 6] * off[2];
        const double* U = &m.ur[12 * tri[node]];
        for (int col = 0; col < 3; ++col)
          m.elOffset.push_back(so[0] * U[3 * col] + so[1] * U[3 * col + 1] + so[2] * U[3 * col + 2]);
      }
      for (double v : S) m.supTr.push_back(v);
      double ss = r.num("stiffscale", 1.0), ms = r.num("massscale", 1.0);
      double a1 = r.num("alpha1", 0.0), a2 = r.num("alpha2", 0.0);
      m.stifScl.push_back(ss);  // temporarily: stiffness scale, replaced below
      m.kDmp.push_back(a2);
      m.C.push_back(ms);        // temporarily: mass scale
      m.C.push_back(a1);        // temporarily: alpha1
      int pid = r.inum("elpropid", 0), pidx = -1;
      for (size_t k = 0; k < props.size(); ++k)
        if (props[k].id == pid) pidx = (int)k;
      if (pidx < 0) { err = "superelement refers to unknown element property"; return -14; }
      elProp.push_back(pidx);
      m.trUnd.resize(24 * (size_t)m.nel, 0.0);
    } else if (nr.name == "triad_undpos") {
      auto it = elIndex.find(r.inum("supelid", 0));
      if (it == elIndex.end()) { err = "undeformed position for unknown superelement"; return -15; }
      int e = it->second, tid = r.inum("triadid", 0), node = -1;
      for (int k = 0; k < 2; ++k)
        if (m.triId[m.elTri[2 * e + k]] == tid) node = k;
      if (node < 0) { err = "undeformed position for unconnected triad"; return -16; }
      auto u = r.nums("undposinsupelsystem");
      // stored transposed in the rotation part (initiateSupElTypeModule.f90:312): file rows -> columns
      double* T = &m.trUnd[24 * (size_t)e + 12 * node];
      for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 3; ++row) {
          size_t k = (size_t)(4 * row + col);
          T[row + 3 * col] = k < u.size() ? u[k] : 0.0;
        }
    } else if (nr.name == "load") {
      auto it = triIndex.find(r.inum("triadid", 0));
      if (it == triIndex.end()) { err = "load on unknown triad"; return -17; }
      int dof = r.inum("ldof", 0);
      if (dof < 1 || dof > m.triNdof[it->second]) { err = "load DOF must be 1..6"; return -18; }
      if (m.dofDep[m.triFirstDof[it->second]] >= 0) { err = "loads on a joint's dependent triad are not supported"; return -79; }
      int eq = m.meqn[m.triFirstDof[it->second] + dof - 1];
      const int eid = r.inum("loadengineid", 0);
      if (eid > 0) {
        auto en = engines.find(eid);
        if (en == engines.end()) { err = "load refers to unknown engine"; return -19; }
        if (eq >= 0)
          engineLoads[eq].push_back({r.num("f0", 0.0), r.num("f1", 0.0), en->second.eA, en->second.eB,
                                     (double)en->second.ch, en->second.sine[0], en->second.sine[1],
                                     en->second.sine[2], en->second.sine[3]});
      } else if (eq >= 0) {
        m.qext[eq] += r.num("f0", 0.0);
      }
    }
  }
  m.ldPtr.assign(1, 0);
  for (auto& kv : engineLoads) {
    m.ldEq.push_back(kv.first);
    for (auto& l : kv.second) {
      m.ldF0.push_back(l[0]); m.ldF1.push_back(l[1]); m.ldEA.push_back(l[2]); m.ldEB.push_back(l[3]);
      m.ldCh.push_back((int)l[4]);
      for (int k = 5; k < 9; ++k) m.ldSin.push_back(l[k]);
    }
    m.ldPtr.push_back((int)m.ldF0.size());
  }
  // axial springs (SPRING_ELEMENT + SPRING_BASE) first, then axial dampers (DAMPER)
  std::map<int, const NmlRecord*> springBase;
  for (const NmlRecord& nr : recs)
    if (nr.name == "spring_base") springBase[Rec{nr}.inum("id", 0)] = &nr;
  for (int pass = 0; pass < 2; ++pass)
    for (const NmlRecord& nr : recs) {
      Rec r{nr};
      int t[2];
      if (pass == 0 && nr.name == "spring_element") {
        auto tids = r.nums("triadids");
        auto sb = r.nums("springbaseid");
        int nb = 0;
        for (double v : sb) nb += v > 0.0;
        if (tids.size() < 2 || tids[1] <= 0.0 || (tids.size() > 2 && tids[2] > 0.0) || nb != 1 || sb[0] <= 0.0) {
          err = "only axial springs between two triads with one base spring are supported";
          return -40;
        }
        auto b = springBase.find((int)std::lround(sb[0]));
        if (b == springBase.end()) { err = "spring refers to unknown SPRING_BASE"; return -43; }
        Rec br{*b->second};
        for (const char* key : {"stifffuncid", "forcefuncid", "lengthengineid", "stiffscaleengineposid",
                                "stiffscaleenginenegid", "springfailureid", "springyieldid"})
          if (br.inum(key, 0) > 0) { err = "only constant linear springs are supported"; return -42; }
        for (int k = 0; k < 2; ++k) {
          auto it = triIndex.find((int)std::lround(tids[k]));
          if (it == triIndex.end()) { err = "spring refers to unknown triad"; return -41; }
          t[k] = it->second;
        }
        m.axKind.push_back(0);
        m.axS0.push_back(br.num("s0", 0.0));
        m.axL0.push_back(br.num("l0", 0.0));
        m.axAlpha2.push_back(r.num("alpha2", 0.0));
        m.axD0.push_back(0.0);
      } else if (pass == 1 && nr.name == "damper") {
        int id1 = r.inum("triad1id", 0), id2 = r.inum("triad2id", 0);
        if (id1 <= 0 || id2 <= 0) { err = "only axial dampers between two triads are supported"; return -44; }
        if (r.inum("coeffscaleengineid", 0) > 0 || r.inum("coefffuncid", 0) > 0 || r.inum("forcefuncid", 0) > 0) {
          err = "only constant linear dampers are supported";
          return -45;
        }
        auto i1 = triIndex.find(id1), i2 = triIndex.find(id2);
        if (i1 == triIndex.end() || i2 == triIndex.end()) { err = "damper refers to unknown triad"; return -46; }
        t[0] = i1->second;
        t[1] = i2->second;
        // the triad with most DOFs is triad 1 (initiateDamperTypeModule.f90:160-165)
        if (m.triNdof[t[0]] < m.triNdof[t[1]]) std::swap(t[0], t[1]);
        m.axKind.push_back(1);
        m.axS0.push_back(0.0);
        m.axL0.push_back(0.0);
        m.axAlpha2.push_back(0.0);
        m.axD0.push_back(r.num("d0", 0.0));
      } else {
        continue;
      }
      for (int k = 0; k < 2; ++k) {
        if (m.triNdof[t[k]] < 3) { err = "axial element triads need translational DOFs"; return -47; }
        if (m.dofDep[m.triFirstDof[t[k]]] >= 0) {
          err = "springs and dampers on a joint's dependent triad are not supported";
          return -79;
        }
        m.axTri.push_back(t[k]);
      }
      m.nax++;
    }
  // element matrices, damping, scaling, corotation initialisation
  std::vector<double> tmpC = m.C;
  m.K.assign(144 * (size_t)m.nel, 0.0);
  m.M.assign(144 * (size_t)m.nel, 0.0);
  m.C.assign(144 * (size_t)m.nel, 0.0);
  m.fg.assign(36 * (size_t)m.nel, 0.0);
  m.triRelSup.assign(12 * (size_t)m.nel, 0.0);
  m.hasC.assign(m.nel, 0);
  m.hasVld.assign(m.nel, 0);
  for (int e = 0; e < m.nel; ++e) {
    double* K = &m.K[144 * (size_t)e];
    double* M = &m.M[144 * (size_t)e];
    double* C = &m.C[144 * (size_t)e];
    double* fg = &m.fg[36 * (size_t)e];
    const double* und = &m.trUnd[24 * (size_t)e];
    if (int rc = beamMatrices(props[elProp[e]], und, und + 12, K, M, fg, err)) return rc;
    double ss = m.stifScl[e], ms = tmpC[2 * e], a1 = tmpC[2 * e + 1], a2 = m.kDmp[e];
    bool damp = a1 > 0.0 || a2 > 0.0;
    if (damp) {
      for (int k = 0; k < 144; ++k) C[k] = a1 * M[k] + a2 * K[k];
      m.hasC[e] = 1;
    }
    if (std::fabs(ss - 1.0) > 1.0e-16)
      for (int k = 0; k < 144; ++k) K[k] *= ss;
    if (std::fabs(ms - 1.0) > 1.0e-16) {
      for (int k = 0; k < 144; ++k) M[k] *= ms;
      for (int k = 0; k < 36; ++k) fg[k] *= ms;
    }
    if (damp && std::fabs(ss - 1.0) > 1.0e-16) a2 /= ss;
    m.kDmp[e] = a2;
    m.stifScl[e] = 1.0;
    m.hasVld[e] = (a2 > 0.0 && c.stiffDampFiltering > 0) ? 1 : 0;
    // triangle frame through the reference points (supElTypeModule.f90:912-950, stat = 1)
    double pts[3][3];
    for (int j = 0; j < 3; ++j) {
      const double* U = &m.ur[12 * m.elTri[2 * e + m.elRef[3 * e + j]]];
      const double* o = &m.elOffset[9 * (size_t)e + 3 * j];
      for (int q = 0; q < 3; ++q) pts[j][q] = U[q] * o[0] + U[q + 3] * o[1] + U[q + 6] * o[2] + U[q + 9];
    }
    double tri[12], inv[12];
    if (frameFrom3Points(pts[0], pts[1], pts[2], tri)) { err = "cannot build corotated frame"; return -22; }
    inverse34(tri, inv);
    compose34(inv, &m.supTr[12 * (size_t)e], &m.triRelSup[12 * (size_t)e]);
  }
  // reduced parts: matrices from their files, structural damping with the
  // generalized DOFs' own factors (computeStructDamping,
  // initiateSupElTypeModule.f90:740-780) on the unscaled matrices, scaling,
  // corotated frame initialisation
  const std::string fsiFile = o.s("fsifile");
  for (int p = 0; p < m.npart; ++p) {
    const int nt = m.pNtri[p], ng = m.pNgen[p], n = 6 * nt + ng, nd = 6 * nt;
    const size_t nn = (size_t)n * n;
    if (n > 96) { err = "parts with more than 96 DOFs (6 per triad + generalized DOFs) are not supported"; return -10; }
    m.pMatOff.push_back((int64_t)m.pK.size());
    m.pVecOff.push_back(p == 0 ? 0 : m.pVecOff[p - 1] + 6 * m.pNtri[p - 1] + m.pNgen[p - 1]);
    m.pGenOff.push_back(p == 0 ? 0 : m.pGenOff[p - 1] + m.pNgen[p - 1]);
    std::vector<double> K, M, fg(3 * (size_t)n, 0.0), C(nn, 0.0);
    if (int rc = readMatrixFile(partFiles[p][0], fsiFile, "stiffness matrix", nn, K, err)) return rc;
    if (int rc = readMatrixFile(partFiles[p][1], fsiFile, "mass matrix", nn, M, err)) return rc;
    if (!partFiles[p][2].empty())
      if (int rc = readMatrixFile(partFiles[p][2], fsiFile, "gravity force vectors", 3 * (size_t)n, fg, err)) return rc;
    const double ss = partScale[p][0], ms = partScale[p][1], a1 = partScale[p][2];
    double a2 = partScale[p][3];
    std::vector<double>& a3 = partA3[p];
    std::vector<double>& a4 = partA4[p];
    bool any3 = false, any4 = false;
    for (int g = 0; g < ng; ++g) {
      any3 = any3 || a3[g] > 0.0;
      any4 = any4 || a4[g] > 0.0;
    }
    for (int g = 0; g < ng; ++g) {
      if (!any3) a3[g] = a1;
      if (!any4) a4[g] = a2;
    }
    const bool damp = a1 > 0.0 || a2 > 0.0 || any3 || any4;
    if (damp) {
      for (size_t k = 0; k < nn; ++k) C[k] = a1 * M[k] + a2 * K[k];
      for (int g = 0; g < ng; ++g) {
        const int j = nd + g;
        const double d3 = a3[g] - a1, d4 = a4[g] - a2;
        if (std::fabs(d3) > 1.0e-16) {
          C[j + (size_t)n * j] += d3 * M[j + (size_t)n * j];
          for (int i = 0; i < nd; ++i) C[i + (size_t)n * j] += d3 * M[i + (size_t)n * j];
          for (int i = 0; i < nd; ++i) C[j + (size_t)n * i] += d3 * M[j + (size_t)n * i];
        }
        if (std::fabs(d4) > 1.0e-16) C[j + (size_t)n * j] += d4 * K[j + (size_t)n * j];
      }
    }
    if (std::fabs(ss - 1.0) > 1.0e-16)
      for (size_t k = 0; k < nn; ++k) K[k] *= ss;
    if (std::fabs(ms - 1.0) > 1.0e-16) {
      for (size_t k = 0; k < nn; ++k) M[k] *= ms;
      for (double& v : fg) v *= ms;
    }
    if (damp && std::fabs(ss - 1.0) > 1.0e-16) a2 /= ss;
    m.pK.insert(m.pK.end(), K.begin(), K.end());
    m.pM.insert(m.pM.end(), M.begin(), M.end());
    m.pC.insert(m.pC.end(), C.begin(), C.end());
    m.pFg.insert(m.pFg.end(), fg.begin(), fg.end());
    m.pStifScl.push_back(1.0);
    m.pKDmp.push_back(a2);
    m.pHasC.push_back(damp ? 1 : 0);
    m.pHasVld.push_back((a2 > 0.0 && c.stiffDampFiltering > 0) ? 1 : 0);
    double pts[3][3];
    for (int j = 0; j < 3; ++j) {
      const double* U = &m.ur[12 * (size_t)m.pTri[m.pTriOff[p] + m.pRef[3 * p + j]]];
      const double* of = &m.pOffset[9 * (size_t)p + 3 * j];
      for (int q = 0; q < 3; ++q) pts[j][q] = U[q] * of[0] + U[q + 3] * of[1] + U[q + 6] * of[2] + U[q + 9];
    }
    double tri[12], inv[12], rel[12];
    if (frameFrom3Points(pts[0], pts[1], pts[2], tri)) { err = "cannot build a part's corotated frame"; return -22; }
    inverse34(tri, inv);
    compose34(inv, &m.pSupTr[12 * (size_t)p], rel);
    for (double v : rel) m.pTriRelSup.push_back(v);
  }
  if (m.npart > 0 && c.tQStatic > c.tStart && c.fixedIt == -1) {
    err = "parts together with pure linear quasi-static steps are not supported";
    return -77;
  }
  // element equation lists
  m.elEq.resize(12 * (size_t)m.nel);
  for (int e = 0; e < m.nel; ++e)
    for (int n = 0; n < 2; ++n)
      for (int d = 0; d < 6; ++d) m.elEq[12 * e + 6 * n + d] = m.meqn[m.triFirstDof[m.elTri[2 * e + n]] + d];
  m.axEq.resize(6 * (size_t)m.nax);
  for (int a = 0; a < m.nax; ++a)
    for (int n = 0; n < 2; ++n)
      for (int d = 0; d < 3; ++d) m.axEq[6 * a + 3 * n + d] = m.meqn[m.triFirstDof[m.axTri[2 * a + n]] + d];
  // elements with a joint's dependent triad: expanded DOFs (the master's DOFs
  // and the joint DOFs in place of the dependent triad's; asmSparse with
  // MEEN < 0, sysMatrixTypeModule.f90:2099-2259)
  m.elCx.assign(m.nel, -1);
  for (int e = 0; e < m.nel; ++e) {
    const int ta = m.elTri[2 * e], tb = m.elTri[2 * e + 1];
    if (m.dofDep[m.triFirstDof[ta]] < 0 && m.dofDep[m.triFirstDof[tb]] < 0) continue;
    m.elCx[e] = (int)m.cxEl.size();
    m.cxEl.push_back(e);
    m.cxEqOff.push_back((int)m.cxEq.size());
    for (int n = 0; n < 2; ++n) {
      const int t = m.elTri[2 * e + n], dd = m.dofDep[m.triFirstDof[t]];
      if (dd >= 0) {
        const int j = dd / 6;
        for (int col = 0; col < m.jNM[j] + m.jNdof[j]; ++col) m.cxEq.push_back(m.jColEq[12 * j + col]);
      } else {
        for (int d = 0; d < 6; ++d) m.cxEq.push_back(m.meqn[m.triFirstDof[t] + d]);
      }
    }
    const int nx = (int)m.cxEq.size() - m.cxEqOff.back();
    m.cxNx.push_back(nx);
    m.cxMatOff.push_back(m.cxMatSize);
    m.cxVecOff.push_back(m.cxVecSize);
    m.cxMatSize += nx * nx;
    m.cxVecSize += 4 * nx;
  }
  m.cxEqOff.push_back((int)m.cxEq.size());
  // reduced parts in expanded form, after the beam elements above
  for (int p = 0; p < m.npart; ++p) {
    m.pXEqOff.push_back((int)m.cxEq.size());
    for (int k = 0; k < m.pNtri[p]; ++k) {
      const int t = m.pTri[m.pTriOff[p] + k], dd = m.dofDep[m.triFirstDof[t]];
      if (dd >= 0) {
        const int j = dd / 6;
        for (int col = 0; col < m.jNM[j] + m.jNdof[j]; ++col) m.cxEq.push_back(m.jColEq[12 * j + col]);
      } else {
        for (int d = 0; d < 6; ++d) m.cxEq.push_back(m.meqn[m.triFirstDof[t] + d]);
      }
    }
    for (int g = 0; g < m.pNgen[p]; ++g) m.cxEq.push_back(m.meqn[m.pGenFirstDof[p] + g]);
    const int nx = (int)m.cxEq.size() - m.pXEqOff.back();
    m.pNx.push_back(nx);
    m.pXMatOff.push_back(m.cxMatSize);
    m.pXVecOff.push_back(m.cxVecSize);
    if ((int64_t)m.cxMatSize + (int64_t)nx * nx >= INT_MAX / 4) { err = "too many part matrix entries"; return -10; }
    m.cxMatSize += nx * nx;
    m.cxVecSize += 4 * nx;
  }
  m.pXEqOff.push_back((int)m.cxEq.size());
  const int xMatBase = 144 * m.nel + 36 * m.nax, xVecBase = 12 * m.nel + 6 * m.nax;
  // full symmetric CSR pattern (union of element cliques, diagonal always present)
  std::vector<std::vector<int>> rows(m.neq);
  for (int i = 0; i < m.neq; ++i) rows[i].push_back(i);
  auto clique = [&](const int* q, int n) {
    for (int i = 0; i < n; ++i) {
      if (q[i] < 0) continue;
      for (int j = 0; j < n; ++j)
        if (q[j] >= 0) rows[q[i]].push_back(q[j]);
    }
  };
  for (int e = 0; e < m.nel; ++e) {
    const int c = m.elCx[e];
    if (c < 0) clique(&m.elEq[12 * e], 12);
    else clique(&m.cxEq[m.cxEqOff[c]], m.cxNx[c]);
  }
  for (int p = 0; p < m.npart; ++p) clique(&m.cxEq[m.pXEqOff[p]], m.pNx[p]);
  for (int a = 0; a < m.nax; ++a) clique(&m.axEq[6 * a], 6);
  m.rowPtr.assign(m.neq + 1, 0);
  for (int i = 0; i < m.neq; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    rows[i].erase(std::unique(rows[i].begin(), rows[i].end()), rows[i].end());
    m.rowPtr[i + 1] = m.rowPtr[i] + (int)rows[i].size();
  }
  m.colInd.reserve(m.rowPtr[m.neq]);
  for (int i = 0; i < m.neq; ++i) m.colInd.insert(m.colInd.end(), rows[i].begin(), rows[i].end());
  // slot <- (element, entry) lists, in element order (deterministic summation order)
  // (slot, source) pairs in visiting order, then a stable counting sort by
  // slot: each slot's list keeps the visiting order
  std::vector<std::pair<int, int>> slotPairs;
  slotPairs.reserve((size_t)144 * m.nel + (size_t)36 * m.nax);
  for (int e = 0; e < m.nel; ++e) {
    const int c = m.elCx[e];
    const int n = c < 0 ? 12 : m.cxNx[c];
    const int* q = c < 0 ? &m.elEq[12 * e] : &m.cxEq[m.cxEqOff[c]];
    for (int i = 0; i < n; ++i) {
      if (q[i] < 0) continue;
      const int* b = &m.colInd[m.rowPtr[q[i]]];
      const int* en = &m.colInd[0] + m.rowPtr[q[i] + 1];
      for (int j = 0; j < n; ++j) {
        if (q[j] < 0) continue;
        int slot = (int)(std::lower_bound(b, en, q[j]) - &m.colInd[0]);
        slotPairs.push_back({slot, c < 0 ? 144 * e + i + 12 * j : xMatBase + m.cxMatOff[c] + i + n * j});
      }
    }
  }
  for (int p = 0; p < m.npart; ++p) {
    const int n = m.pNx[p];
    const int* q = &m.cxEq[m.pXEqOff[p]];
    for (int i = 0; i < n; ++i) {
      if (q[i] < 0) continue;
      const int* b = &m.colInd[m.rowPtr[q[i]]];
      const int* en = &m.colInd[0] + m.rowPtr[q[i] + 1];
      for (int j = 0; j < n; ++j) {
        if (q[j] < 0) continue;
        int slot = (int)(std::lower_bound(b, en, q[j]) - &m.colInd[0]);
        slotPairs.push_back({slot, xMatBase + m.pXMatOff[p] + i + n * j});
      }
    }
  }
  for (int a = 0; a < m.nax; ++a) {  // springs, then dampers (BuildNewtonMat order)
    const int* q = &m.axEq[6 * a];
    for (int i = 0; i < 6; ++i) {
      if (q[i] < 0) continue;
      const int* b = &m.colInd[m.rowPtr[q[i]]];
      const int* en = &m.colInd[0] + m.rowPtr[q[i] + 1];
      for (int j = 0; j < 6; ++j) {
        if (q[j] < 0) continue;
        int slot = (int)(std::lower_bound(b, en, q[j]) - &m.colInd[0]);
        slotPairs.push_back({slot, 144 * m.nel + 36 * a + i + 6 * j});
      }
    }
  }
  m.slotPtr.assign(m.colInd.size() + 1, 0);
  for (const auto& sp : slotPairs) ++m.slotPtr[sp.first + 1];
  for (size_t s = 0; s < m.colInd.size(); ++s) m.slotPtr[s + 1] += m.slotPtr[s];
  m.slotSrc.assign(slotPairs.size(), 0);
  {
    std::vector<int> cur(m.slotPtr.begin(), m.slotPtr.end() - 1);
    for (const auto& sp : slotPairs) m.slotSrc[cur[sp.first]++] = sp.second;
  }
  // equation <- (element, local DOF) lists
  std::vector<std::vector<int>> eqList(m.neq);
  for (int e = 0; e < m.nel; ++e) {
    const int c = m.elCx[e];
    if (c < 0) {
      for (int i = 0; i < 12; ++i)
        if (m.elEq[12 * e + i] >= 0) eqList[m.elEq[12 * e + i]].push_back(12 * e + i);
    } else {
      for (int i = 0; i < m.cxNx[c]; ++i) {
        const int q = m.cxEq[m.cxEqOff[c] + i];
        if (q >= 0) eqList[q].push_back(xVecBase + m.cxVecOff[c] + 4 * i);
      }
    }
  }
  for (int p = 0; p < m.npart; ++p)
    for (int i = 0; i < m.pNx[p]; ++i) {
      const int q = m.cxEq[m.pXEqOff[p] + i];
      if (q >= 0) eqList[q].push_back(xVecBase + m.pXVecOff[p] + 4 * i);
    }
  for (int a = 0; a < m.nax; ++a)
    for (int i = 0; i < 6; ++i)
      if (m.axEq[6 * a + i] >= 0) eqList[m.axEq[6 * a + i]].push_back(12 * m.nel + 6 * a + i);
  m.eqPtr.assign(m.neq + 1, 0);
  for (int i = 0; i < m.neq; ++i) m.eqPtr[i + 1] = m.eqPtr[i] + (int)eqList[i].size();
  for (auto& l : eqList) m.eqSrc.insert(m.eqSrc.end(), l.begin(), l.end());
  // prescribed-DOF terms moved to the right-hand side (asmSparse with a constant
  // term, sysMatrixTypeModule.f90:2099-2259): element order, then prescribed row
  std::vector<std::vector<std::pair<int, int>>> mrList(m.neq);
  for (int e = 0; e < m.nel; ++e) {
    const int* q = &m.elEq[12 * e];
    for (int i = 0; i < 12; ++i) {
      if (q[i] > -2) continue;
      for (int j = 0; j < 12; ++j)
        if (q[j] >= 0) mrList[q[j]].push_back({144 * e + i + 12 * j, -2 - q[i]});
    }
  }
  for (int p = 0; p < m.npart; ++p) {
    const int n = m.pNx[p];
    const int* q = &m.cxEq[m.pXEqOff[p]];
    for (int i = 0; i < n; ++i) {
      if (q[i] > -2) continue;
      for (int j = 0; j < n; ++j)
        if (q[j] >= 0) mrList[q[j]].push_back({xMatBase + m.pXMatOff[p] + i + n * j, -2 - q[i]});
    }
  }
  for (int a = 0; a < m.nax; ++a) {
    const int* q = &m.axEq[6 * a];
    for (int i = 0; i < 6; ++i) {
      if (q[i] > -2) continue;
      for (int j = 0; j < 6; ++j)
        if (q[j] >= 0) mrList[q[j]].push_back({144 * m.nel + 36 * a + i + 6 * j, -2 - q[i]});
    }
  }
  m.mrPtr.assign(1, 0);
  for (int i = 0; i < m.neq; ++i) {
    if (mrList[i].empty()) continue;
    m.mrEq.push_back(i);
    for (auto& pr : mrList[i]) {
      m.mrSrc.push_back(pr.first);
      m.mrMot.push_back(pr.second);
    }
    m.mrPtr.push_back((int)m.mrSrc.size());
  }
  return symbolicAnalysis(m, err);
}

}  // namespace fgpu
