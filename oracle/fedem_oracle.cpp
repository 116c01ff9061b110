// fedem_oracle.cpp -- CPU oracle (FP64 restatement) of the FEDEM dynamics
// solver's implicit HHT-alpha/Newmark Newton time step for beam models.
//
// TEST INFRASTRUCTURE ONLY: this file is the parity checker for the CUDA
// solver and the timed CPU baseline.  It is never linked into the product.
//
// Every routine names the reference routine it restates (file:line, paths
// relative to the fedem-solvers source tree).  The sparse LDL^T of the absent
// SAM/SPR library is replaced by a skyline (profile) LDL^T over the equations
// in their natural (DOF) order, the same storage as the reference's own
// -skylinesolver option (asmExtensionModule.f90:1282-1294, ADDEM1).

#include "fedem_oracle.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

// ===========================================================================
// Namelist subset reader for the solver input file (.fsi).
// Follows the records read by initiateTriadTypeModule.f90, supElTypeModule.f90:1301-1365,
// finiteElementModule.f90:151, forceTypeModule.f90:157, mechanismTypeModule.f90.
// ===========================================================================

struct Record {
  std::string name;
  std::map<std::string, std::vector<std::string>> kv;
  const std::vector<std::string>* get(const char* key) const {
    auto it = kv.find(key);
    return it == kv.end() ? nullptr : &it->second;
  }
  bool has(const char* key) const { return kv.count(key) > 0; }
  double d(const char* key, double def = 0.0) const {
    const auto* v = get(key);
    if (!v || v->empty()) return def;
    return toD((*v)[0]);
  }
  int i(const char* key, int def = 0) const {
    const auto* v = get(key);
    if (!v || v->empty()) return def;
    return (int)std::lround(toD((*v)[0]));
  }
  std::vector<double> dv(const char* key) const {
    std::vector<double> out;
    const auto* v = get(key);
    if (v)
      for (const auto& s : *v) out.push_back(toD(s));
    return out;
  }
  std::string s(const char* key) const {
    const auto* v = get(key);
    if (!v || v->empty()) return std::string();
    return (*v)[0];
  }
  static double toD(std::string t) {
    for (auto& c : t)
      if (c == 'd' || c == 'D') c = 'e';
    return std::strtod(t.c_str(), nullptr);
  }
};

static std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// Splits the text into &NAME ... / records with key = value lists.
// Values may be numbers, quoted strings or logicals; "n*v" repeats v n times.
static std::vector<Record> parseNamelists(const char* text) {
  std::vector<Record> recs;
  const char* p = text;
  const char* end = text + std::strlen(text);
  while (p < end) {
    // find '&' at the start of a token outside any record
    const char* amp = std::strchr(p, '&');
    if (!amp) break;
    p = amp + 1;
    const char* q = p;
    while (q < end && (std::isalnum((unsigned char)*q) || *q == '_')) ++q;
    Record rec;
    rec.name = lower(std::string(p, q));
    p = q;
    // tokenize until '/'
    std::vector<std::string> toks;
    std::vector<int> kinds;  // 0 word, 1 '=', 2 string
    bool closed = false;
    while (p < end && !closed) {
      char c = *p;
      if (std::isspace((unsigned char)c) || c == ',') { ++p; continue; }
      if (c == '!') { while (p < end && *p != '\n') ++p; continue; }
      if (c == '/') { ++p; closed = true; break; }
      if (c == '=') { toks.emplace_back("="); kinds.push_back(1); ++p; continue; }
      if (c == '\'' || c == '"') {
        char qc = c;
        const char* s0 = ++p;
        while (p < end && *p != qc) ++p;
        toks.emplace_back(s0, p);
        kinds.push_back(2);
        if (p < end) ++p;
        continue;
      }
      const char* s0 = p;
      while (p < end && !std::isspace((unsigned char)*p) && *p != ',' && *p != '=' &&
             *p != '/' && *p != '\'' && *p != '"')
        ++p;
      toks.emplace_back(s0, p);
      kinds.push_back(0);
    }
    // assemble key = values
    std::string key;
    for (size_t k = 0; k < toks.size(); ++k) {
      if (kinds[k] == 0 && k + 1 < toks.size() && kinds[k + 1] == 1) {
        key = lower(toks[k]);
        rec.kv[key];  // create
        ++k;
        continue;
      }
      if (key.empty()) continue;
      if (kinds[k] == 0) {
        const std::string& t = toks[k];
        size_t star = t.find('*');
        if (star != std::string::npos && star > 0) {
          int n = std::atoi(t.substr(0, star).c_str());
          for (int r = 0; r < n; ++r) rec.kv[key].push_back(t.substr(star + 1));
          continue;
        }
      }
      rec.kv[key].push_back(toks[k]);
    }
    recs.push_back(std::move(rec));
  }
  return recs;
}

// ===========================================================================
// Command-line options: -name=value, -name (true), -name- (false), -name+ (true)
// Defaults follow the ADDOPTION table of src/vpmSolver/solverInterface.C:195-554.
// ===========================================================================

struct Options {
  std::map<std::string, std::string> m;
  void parse(int argc, const char* const* argv) {
    for (int k = 0; k < argc; ++k) {
      if (!argv[k]) continue;
      std::string a = argv[k];
      if (a.size() < 2 || a[0] != '-') continue;
      a = a.substr(1);
      size_t eq = a.find('=');
      std::string key, val;
      if (eq != std::string::npos) {
        key = a.substr(0, eq);
        val = a.substr(eq + 1);
        if (val.size() >= 2 && (val.front() == '"' || val.front() == '\'') && val.back() == val.front())
          val = val.substr(1, val.size() - 2);
      } else if (!a.empty() && a.back() == '-') {
        key = a.substr(0, a.size() - 1);
        val = "false";
      } else if (!a.empty() && a.back() == '+') {
        key = a.substr(0, a.size() - 1);
        val = "true";
      } else {
        key = a;
        val = "true";
      }
      m[lower(key)] = val;
    }
  }
  bool has(const char* k) const { return m.count(lower(k)) > 0; }
  double d(const char* k, double def) const {
    auto it = m.find(lower(k));
    return it == m.end() ? def : Record::toD(it->second);
  }
  int i(const char* k, int def) const {
    auto it = m.find(lower(k));
    return it == m.end() ? def : (int)std::lround(Record::toD(it->second));
  }
  bool b(const char* k, bool def) const {
    auto it = m.find(lower(k));
    if (it == m.end()) return def;
    std::string v = lower(it->second);
    return v == "true" || v == "1" || v == "yes" || v == "on" || v == "t";
  }
  std::string s(const char* k) const {
    auto it = m.find(lower(k));
    return it == m.end() ? std::string() : it->second;
  }
};

// ===========================================================================
// 3x4 position matrices T[r][c]: columns 0..2 rotation, column 3 position.
// Restates src/vpmUtilities/manipMatrixModule.f90:287-594.
// ===========================================================================

typedef double M34[3][4];

static void matmul34(const M34 a, const M34 b, M34 out) {  // manipMatrixModule.f90:287
  M34 r;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 4; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += a[i][k] * b[k][j];
      r[i][j] = s;
    }
    r[i][3] += a[i][3];
  }
  std::memcpy(out, r, sizeof(M34));
}

static void invert34(const M34 a, M34 b) {  // manipMatrixModule.f90:426
  M34 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r[i][j] = a[j][i];
  for (int i = 0; i < 3; ++i) r[i][3] = -(r[i][0] * a[0][3] + r[i][1] * a[1][3] + r[i][2] * a[2][3]);
  std::memcpy(b, r, sizeof(M34));
}

static void cross(const double* a, const double* b, double* c) {
  double t0 = a[1] * b[2] - a[2] * b[1];
  double t1 = a[2] * b[0] - a[0] * b[2];
  double t2 = a[0] * b[1] - a[1] * b[0];
  c[0] = t0; c[1] = t1; c[2] = t2;
}

static const double epsDiv0 = 1.0e-16;

// Coordinate system from three points (manipMatrixModule.f90:447-537).
static int trans3P(const double* p1, const double* p2, const double* p3, M34 tr) {
  double c1[3], c2[3], c3[3];
  for (int k = 0; k < 3; ++k) { c1[k] = p2[k] - p1[k]; c2[k] = p3[k] - p1[k]; }
  cross(c1, c2, c3);
  double l1 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
  if (!(l1 > epsDiv0)) return -1;
  double s1 = std::sqrt(l1);
  for (int k = 0; k < 3; ++k) c1[k] /= s1;
  double l3 = c3[0] * c3[0] + c3[1] * c3[1] + c3[2] * c3[2];
  if (!(l3 > epsDiv0)) return -2;
  double s3 = std::sqrt(l3);
  for (int k = 0; k < 3; ++k) c3[k] /= s3;
  cross(c3, c1, c2);
  for (int k = 0; k < 3; ++k) {
    tr[k][0] = c1[k]; tr[k][1] = c2[k]; tr[k][2] = c3[k]; tr[k][3] = p1[k];
  }
  return 0;
}

// Local axes from one direction vector (manipMatrixModule.f90:547-594); T[r][c].
static int trans1V(const double* v, double T[3][3]) {
  double sq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  if (!(std::fabs(sq) > epsDiv0)) return -1;
  double s = std::sqrt(sq);
  for (int k = 0; k < 3; ++k) T[k][0] = v[k] / s;
  double c1[3] = {T[0][0], T[1][0], T[2][0]}, c2[3], c3[3];
  if (std::fabs(T[2][0]) > std::fabs(T[1][0])) {
    c2[0] = -T[1][0] * T[0][0];
    c2[1] = T[0][0] * T[0][0] + T[2][0] * T[2][0];
    c2[2] = -T[1][0] * T[2][0];
    double l = std::sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]);
    for (int k = 0; k < 3; ++k) c2[k] /= l;
    cross(c1, c2, c3);
  } else {
    c3[0] = -T[2][0] * T[0][0];
    c3[1] = -T[2][0] * T[1][0];
    c3[2] = T[0][0] * T[0][0] + T[1][0] * T[1][0];
    double l = std::sqrt(c3[0] * c3[0] + c3[1] * c3[1] + c3[2] * c3[2]);
    for (int k = 0; k < 3; ++k) c3[k] /= l;
    cross(c3, c1, c2);
  }
  for (int k = 0; k < 3; ++k) { T[k][1] = c2[k]; T[k][2] = c3[k]; }
  return 0;
}

// Rotation tensor from a rotation vector through a normalised quaternion
// (rotationModule.f90:355-370, vec_to_quat :393-436, quat_to_mat :478-500).
static void vec_to_mat(const double* rv, double R[3][3]) {
  const double epsTh2 = 0.0005;
  double thh = 0.5 * std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double sthh = std::sin(thh), cthh = std::cos(thh);
  double fac;
  if (thh < epsTh2) {
    double f1 = thh / epsTh2;
    fac = f1 * std::sin(epsTh2) / epsTh2 + 1.0 - f1;
  } else {
    fac = sthh / thh;
  }
  double q[4] = {cthh, rv[0] * fac * 0.5, rv[1] * fac * 0.5, rv[2] * fac * 0.5};
  double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) q[k] /= n;
  n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) q[k] /= n;
  R[0][0] = 2.0 * (q[1] * q[1] + q[0] * q[0]) - 1.0;
  R[1][1] = 2.0 * (q[2] * q[2] + q[0] * q[0]) - 1.0;
  R[2][2] = 2.0 * (q[3] * q[3] + q[0] * q[0]) - 1.0;
  R[0][1] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
  R[0][2] = 2.0 * (q[1] * q[3] + q[2] * q[0]);
  R[1][2] = 2.0 * (q[2] * q[3] - q[1] * q[0]);
  R[1][0] = 2.0 * (q[2] * q[1] + q[3] * q[0]);
  R[2][0] = 2.0 * (q[3] * q[1] - q[2] * q[0]);
  R[2][1] = 2.0 * (q[3] * q[2] + q[1] * q[0]);
}

// Re-orthonormalises a rotation tensor via its quaternion
// (rotationModule.f90:549-558, mat_to_quat :447-476, quat_to_mat :478-500).
static void orthonorm3(double R[3][3]) {
  double q[4];
  double tr = R[0][0] + R[1][1] + R[2][2];
  int imax = 0;
  if (R[1][1] > R[imax][imax]) imax = 1;
  if (R[2][2] > R[imax][imax]) imax = 2;
  if (tr > R[imax][imax]) {
    q[0] = std::sqrt(1.0 + tr) * 0.5;
    q[1] = (R[2][1] - R[1][2]) / (4.0 * q[0]);
    q[2] = (R[0][2] - R[2][0]) / (4.0 * q[0]);
    q[3] = (R[1][0] - R[0][1]) / (4.0 * q[0]);
  } else {
    int i = imax, j = (imax + 1) % 3, k = (imax + 2) % 3;
    q[i + 1] = std::sqrt(R[i][i] * 0.5 + (1.0 - tr) * 0.25);
    q[0] = (R[k][j] - R[j][k]) / (4.0 * q[i + 1]);
    q[j + 1] = (R[j][i] + R[i][j]) / (4.0 * q[i + 1]);
    q[k + 1] = (R[k][i] + R[i][k]) / (4.0 * q[i + 1]);
  }
  double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int a = 0; a < 4; ++a) q[a] /= n;
  R[0][0] = 2.0 * (q[1] * q[1] + q[0] * q[0]) - 1.0;
  R[1][1] = 2.0 * (q[2] * q[2] + q[0] * q[0]) - 1.0;
  R[2][2] = 2.0 * (q[3] * q[3] + q[0] * q[0]) - 1.0;
  R[0][1] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
  R[0][2] = 2.0 * (q[1] * q[3] + q[2] * q[0]);
  R[1][2] = 2.0 * (q[2] * q[3] - q[1] * q[0]);
  R[1][0] = 2.0 * (q[2] * q[1] + q[3] * q[0]);
  R[2][0] = 2.0 * (q[3] * q[1] - q[2] * q[0]);
  R[2][1] = 2.0 * (q[3] * q[2] + q[1] * q[0]);
}

// ===========================================================================
// 12-DOF beam element (src/Femlib/beam.f, src/Femlib/beamaux.f).
// Matrices are column-major: A[i + 12*j] == A(i+1,j+1).
// ===========================================================================

#define A12(A, i, j) A[((i) - 1) + 12 * ((j) - 1)]

// Direction cosines, local <- global (beamaux.f:48-104).  C[r][c] == C(r+1,c+1).
static void dcos30(double C[3][3], const double* X, const double* Y, const double* Z) {
  double cx = X[1] - X[0], cy = Y[1] - Y[0], cz = Z[1] - Z[0];
  double ab = std::sqrt(cx * cx + cy * cy + cz * cz);
  C[0][0] = cx / ab; C[0][1] = cy / ab; C[0][2] = cz / ab;
  cx = C[0][2] * (Y[2] - Y[0]) - C[0][1] * (Z[2] - Z[0]);
  cy = C[0][0] * (Z[2] - Z[0]) - C[0][2] * (X[2] - X[0]);
  cz = C[0][1] * (X[2] - X[0]) - C[0][0] * (Y[2] - Y[0]);
  ab = std::sqrt(cx * cx + cy * cy + cz * cz);
  C[1][0] = cx / ab; C[1][1] = cy / ab; C[1][2] = cz / ab;
  cx = C[0][1] * C[1][2] - C[0][2] * C[1][1];
  cy = C[0][2] * C[1][0] - C[0][0] * C[1][2];
  cz = C[0][0] * C[1][1] - C[0][1] * C[1][0];
  ab = std::sqrt(cx * cx + cy * cy + cz * cz);
  C[2][0] = cx / ab; C[2][1] = cy / ab; C[2][2] = cz / ab;
}

// Congruence transformation with a repeated 3x3 block (beamaux.f:106-163).
static void mpro30(double* EK, double C[3][3]) {
  const int M = 12;
  for (int I = 0; I <= M - 3; I += 3)
    for (int J = 0; J <= M - 3; J += 3) {
      double B[3][3] = {{0}};
      for (int IA = 1; IA <= 3; ++IA) {
        int IB = I + IA;
        for (int KA = 1; KA <= 3; ++KA) {
          int JB = J + KA;
          for (int JA = 1; JA <= 3; ++JA) B[JA - 1][IA - 1] += C[KA - 1][JA - 1] * A12(EK, JB, IB);
        }
      }
      for (int IA = 1; IA <= 3; ++IA)
        for (int KA = 1; KA <= 3; ++KA) A12(EK, J + KA, I + IA) = 0.0;
      for (int IA = 1; IA <= 3; ++IA) {
        int IB = I + IA;
        for (int KA = 1; KA <= 3; ++KA) {
          int JB = J + KA;
          for (int JA = 1; JA <= 3; ++JA) A12(EK, JB, IB) += B[KA - 1][JA - 1] * C[JA - 1][IA - 1];
        }
      }
    }
  for (int i = 1; i <= M; ++i)
    for (int j = i; j <= M; ++j) A12(EK, i, j) = A12(EK, j, i);
}

// End points -> eccentric nodal points (beamaux.f:165-201).
static void trix30(double* A, double X1, double Y1, double Z1, double X2, double Y2, double Z2) {
  for (int i = 1; i <= 12; ++i) {
    A12(A, 4, i) += Z1 * A12(A, 2, i) - Y1 * A12(A, 3, i);
    A12(A, 5, i) += -Z1 * A12(A, 1, i) + X1 * A12(A, 3, i);
    A12(A, 6, i) += Y1 * A12(A, 1, i) - X1 * A12(A, 2, i);
    A12(A, 10, i) += Z2 * A12(A, 8, i) - Y2 * A12(A, 9, i);
    A12(A, 11, i) += -Z2 * A12(A, 7, i) + X2 * A12(A, 9, i);
    A12(A, 12, i) += Y2 * A12(A, 7, i) - X2 * A12(A, 8, i);
  }
  for (int i = 1; i <= 12; ++i) {
    A12(A, i, 4) += Z1 * A12(A, i, 2) - Y1 * A12(A, i, 3);
    A12(A, i, 5) += -Z1 * A12(A, i, 1) + X1 * A12(A, i, 3);
    A12(A, i, 6) += Y1 * A12(A, i, 1) - X1 * A12(A, i, 2);
    A12(A, i, 10) += Z2 * A12(A, i, 8) - Y2 * A12(A, i, 9);
    A12(A, i, 11) += -Z2 * A12(A, i, 7) + X2 * A12(A, i, 9);
    A12(A, i, 12) += Y2 * A12(A, i, 7) - X2 * A12(A, i, 8);
  }
}

// Local stiffness matrix (beam.f:619-760, BELS31).
static void bels31(double* EK, double BL, const double* EP, const double* CA, const double* XS) {
  double E = EP[0], G = EP[1], A = EP[2], RIY = EP[3], RIZ = EP[4], RIT = EP[5];
  double CAY = CA[0], CAZ = CA[1], YS = XS[0], ZS = XS[1];
  double EA, EIY, EIZ, ALY, ALZ, GIT;
  if (E < -1.0e-16) {
    EA = A; EIY = RIY; EIZ = RIZ;
    ALY = CAY > 1.0e-16 ? 12.0 * EIY / (CAY * BL * BL) : 0.0;
    ALZ = CAZ > 1.0e-16 ? 12.0 * EIZ / (CAZ * BL * BL) : 0.0;
    GIT = RIT;
  } else {
    EA = E * A; EIY = E * RIY; EIZ = E * RIZ;
    ALY = 12.0 * CAY * EIY / (A * G * BL * BL);
    ALZ = 12.0 * CAZ * EIZ / (A * G * BL * BL);
    GIT = G * RIT;
  }
  for (int k = 0; k < 144; ++k) EK[k] = 0.0;
  A12(EK, 1, 1) = EA / BL;
  A12(EK, 2, 2) = 12. * EIY / (BL * BL * BL * (1. + ALY));
  A12(EK, 3, 3) = 12. * EIZ / (BL * BL * BL * (1. + ALZ));
  A12(EK, 4, 4) = GIT / BL;
  A12(EK, 3, 5) = -.5 * BL * A12(EK, 3, 3);
  A12(EK, 2, 6) = .5 * BL * A12(EK, 2, 2);
  A12(EK, 5, 5) = EIZ * (4. + ALZ) / (BL * (1. + ALZ));
  A12(EK, 6, 6) = EIY * (4. + ALY) / (BL * (1. + ALY));
  A12(EK, 1, 7) = -A12(EK, 1, 1);
  A12(EK, 7, 7) = A12(EK, 1, 1);
  A12(EK, 2, 8) = -A12(EK, 2, 2);
  A12(EK, 6, 8) = -A12(EK, 2, 6);
  A12(EK, 8, 8) = A12(EK, 2, 2);
  A12(EK, 3, 9) = -A12(EK, 3, 3);
  A12(EK, 5, 9) = -A12(EK, 3, 5);
  A12(EK, 9, 9) = A12(EK, 3, 3);
  A12(EK, 4, 10) = -A12(EK, 4, 4);
  A12(EK, 10, 10) = A12(EK, 4, 4);
  A12(EK, 3, 11) = A12(EK, 3, 5);
  A12(EK, 5, 11) = EIZ * (2. - ALZ) / (BL * (1. + ALZ));
  A12(EK, 9, 11) = -A12(EK, 3, 5);
  A12(EK, 11, 11) = A12(EK, 5, 5);
  A12(EK, 2, 12) = A12(EK, 2, 6);
  A12(EK, 6, 12) = EIY * (2. - ALY) / (BL * (1. + ALY));
  A12(EK, 8, 12) = -A12(EK, 2, 6);
  A12(EK, 12, 12) = A12(EK, 6, 6);
  for (int i = 1; i <= 12; ++i)
    for (int j = 1; j <= i; ++j) A12(EK, i, j) = A12(EK, j, i);
  double BE = std::fabs(YS) + std::fabs(ZS);
  double BA = .00001 * std::sqrt(A);
  if (BA - BE < 0.0) {
    for (int i = 1; i <= 12; ++i) {
      A12(EK, 4, i) = A12(EK, 4, i) - ZS * A12(EK, 2, i) + YS * A12(EK, 3, i);
      A12(EK, 10, i) = A12(EK, 10, i) - ZS * A12(EK, 8, i) + YS * A12(EK, 9, i);
    }
    for (int i = 1; i <= 12; ++i) {
      A12(EK, i, 4) = A12(EK, i, 4) - A12(EK, i, 2) * ZS + A12(EK, i, 3) * YS;
      A12(EK, i, 10) = A12(EK, i, 10) - A12(EK, i, 8) * ZS + A12(EK, i, 9) * YS;
    }
  }
}

// Global stiffness matrix (beam.f:11-166, BEAM31, no pins, EFFLEN = PHI = 0).
static int beam31(double* EK, const double* X, const double* Y, const double* Z, const double* EP,
                  const double* CA, const double* XS) {
  double bx = X[1] - X[0], by = Y[1] - Y[0], bz = Z[1] - Z[0];
  double BL = std::sqrt(bx * bx + by * by + bz * bz);
  double BA = 1.0e-6 * (std::fabs(X[0]) + std::fabs(X[1]) + std::fabs(Y[0]) + std::fabs(Y[1]) +
                        std::fabs(Z[0]) + std::fabs(Z[1]));
  if (BL - BA <= 0.0) return -1;
  bx = X[2] - X[0]; by = Y[2] - Y[0]; bz = Z[2] - Z[0];
  if (std::sqrt(bx * bx + by * by + bz * bz) - BA <= 0.0) return -2;
  if (EP[1] <= 1.0e-16 || EP[2] <= 1.0e-16) return -3;
  double T2[3][3];
  dcos30(T2, X, Y, Z);
  bels31(EK, BL, EP, CA, XS);
  mpro30(EK, T2);
  trix30(EK, X[3] - X[0], Y[3] - Y[0], Z[3] - Z[0], X[4] - X[1], Y[4] - Y[1], Z[4] - Z[1]);
  return 0;
}

// Consistent mass matrix (beam.f:396-576, BEAM35 with IOP=3, no pins).
static void beam35(double* EM, const double* X, const double* Y, const double* Z, double A,
                   double RHO, double RIX) {
  for (int k = 0; k < 144; ++k) EM[k] = 0.0;
  double bx = X[1] - X[0], by = Y[1] - Y[0], bz = Z[1] - Z[0];
  double BL = std::sqrt(bx * bx + by * by + bz * bz);
  double AM = BL * A * RHO;
  double AM2 = BL * AM;
  double AM3 = BL * AM2;
  double RM = RIX * RHO;
  A12(EM, 1, 1) = AM / 3.;
  A12(EM, 1, 7) = AM / 6.;
  A12(EM, 2, 2) = 13. * AM / 35.;
  A12(EM, 2, 6) = 11. * AM2 / 210.;
  A12(EM, 2, 8) = 9. * AM / 70.;
  A12(EM, 2, 12) = -13. * AM2 / 420.;
  A12(EM, 3, 3) = A12(EM, 2, 2);
  A12(EM, 3, 5) = -A12(EM, 2, 6);
  A12(EM, 3, 9) = A12(EM, 2, 8);
  A12(EM, 3, 11) = -A12(EM, 2, 12);
  A12(EM, 4, 4) = BL * RM / 3.;
  A12(EM, 4, 10) = BL * RM / 6.;
  A12(EM, 5, 5) = AM3 / 105.;
  A12(EM, 5, 9) = A12(EM, 2, 12);
  A12(EM, 5, 11) = -AM3 / 140.;
  A12(EM, 6, 6) = A12(EM, 5, 5);
  A12(EM, 6, 8) = A12(EM, 3, 11);
  A12(EM, 6, 12) = A12(EM, 5, 11);
  A12(EM, 7, 7) = A12(EM, 1, 1);
  A12(EM, 8, 8) = A12(EM, 2, 2);
  A12(EM, 8, 12) = A12(EM, 3, 5);
  A12(EM, 9, 9) = A12(EM, 8, 8);
  A12(EM, 9, 11) = A12(EM, 2, 6);
  A12(EM, 10, 10) = A12(EM, 4, 4);
  A12(EM, 11, 11) = A12(EM, 5, 5);
  A12(EM, 12, 12) = A12(EM, 6, 6);
  for (int i = 1; i <= 12; ++i)
    for (int j = i; j <= 12; ++j) A12(EM, j, i) = A12(EM, i, j);
  double T2[3][3];
  dcos30(T2, X, Y, Z);
  mpro30(EM, T2);
  trix30(EM, X[3] - X[0], Y[3] - Y[0], Z[3] - Z[0], X[4] - X[1], Y[4] - Y[1], Z[4] - Z[1]);
}

// ===========================================================================
// Model data
// ===========================================================================

struct Triad {
  int id = 0;
  int nDOFs = 6;
  M34 ur, urPrev;
  int BC[6] = {1, 1, 1, 1, 1, 1};
  int firstDof = -1;  // 0-based index into the DOF vectors (MADOF)
};

struct Prop {
  int id = 0;
  double geo[8] = {0};
  double mat[4] = {0};
  double orient[3] = {0};
};

// Superelement (SupElType, supElTypeModule.f90): nTri triads with six DOFs
// each, then nGen generalized (component-mode) DOFs; n = 6 nTri + nGen.  A
// beam is the case nTri = 2, nGen = 0 with matrices from its cross section;
// a reduced part reads K, M and the gravity force vectors from files.
struct Elem {
  int id = 0;
  int nTri = 2, nGen = 0, n = 12;
  std::vector<int> tri;       // triad indices
  int ref[3] = {0, 0, 0};     // local node index of the three reference triads
  double offset[3][3];        // reference point offsets, in triad axes
  M34 supTr, supTrPrev, triRelSup;
  std::vector<double> TrUnd;  // undeformed triad positions, 12 per triad (3x4 row-major)
  std::vector<double> K, M, C, N;  // n x n column-major
  std::vector<double> fg;          // n x 3 column-major gravity force vectors
  bool hasC = false, hasVld = false;
  double stiffScale = 1.0, massScale = 1.0, alpha1 = 0.0, alpha2 = 0.0;
  std::vector<double> alpha3, alpha4;  // damping factors of the generalized DOFs
  double stifScl = 1.0, kDmp = 0.0;
  std::vector<double> finit, finitPrev, uld, uldd, vld;  // vld: the 6 nTri triad DOFs
  std::vector<double> FS, FD, FI, Q;
  std::vector<double> genUr, genUrPrev;  // generalized DOF values (genDOFs%ur)
  std::vector<int> genBC;
  int genFirstDof = -1;  // first generalized DOF in the DOF vectors
  int prop = -1;         // beam property index (elPropId), -1 for a reduced part
  std::string files[3];  // stiffness, mass, gravity force matrix files
  double tu(int i, int r, int c) const { return TrUnd[12 * i + 4 * r + c]; }
  void allocate() {
    n = 6 * nTri + nGen;
    K.assign((size_t)n * n, 0.0);
    M.assign((size_t)n * n, 0.0);
    C.assign((size_t)n * n, 0.0);
    N.assign((size_t)n * n, 0.0);
    fg.assign((size_t)n * 3, 0.0);
    for (auto* v : {&finit, &finitPrev, &uld, &uldd, &FS, &FD, &FI, &Q}) v->assign(n, 0.0);
    vld.assign(6 * nTri, 0.0);
    genUr.assign(nGen, 0.0);
    genUrPrev.assign(nGen, 0.0);
  }
};

struct Load {
  int triad = -1;
  int dof = 0;  // 1..6 system DOF
  double f0 = 0.0, f1 = 0.0;
  int engine = -1;
  double F = 0.0;
};

// General functions (functionTypeModule / engineRoutinesModule subset):
// engine value = f(sensor value); sensor TIME gives the physical time;
// function SCALE gives realData(1) * x; no function gives x.
struct Func { int id = 0; std::string type; std::vector<double> real; };
struct Sensor { int id = 0; std::string type; };
struct EngineF { int id = 0; int func = -1; int sensor = -1; };

// Prescribed motion (motionTypeModule.f90; motionRoutinesModule.f90:58-193)
struct Motion {
  int triad = -1, dof = 0;
  double d0 = 0.0, d1 = 0.0;
  int engine = -1;
  double D = 0.0;  // current prescribed value
  int iceq = 0;    // constraint equation (1-based)
};

// Axial spring (SPRING_ELEMENT with two triads and one SPRING_BASE of
// constant stiffness s0 and stress-free length l0) or axial damper (DAMPER
// between two triads, coefficient d0): springRoutinesModule.f90:200-239,
// 551-742, 872-1124; damperRoutinesModule.f90:54-376.  Forces act along the
// current direction n from triad 1 to triad 2 on the translational DOFs.
struct Axial {
  int kind = 0;  // 0 spring, 1 damper
  int tri[2] = {-1, -1};
  double s0 = 0.0, l0 = 0.0, alpha2 = 0.0, d0 = 0.0;
  double n[3] = {0, 0, 0}, L = 0.0, F = 0.0;
  double FS[6] = {0, 0, 0, 0, 0, 0}, FD[6] = {0, 0, 0, 0, 0, 0};
};

// Master-slave joint with one master triad (MasterSlaveJointTypeModule): the
// slave triad's DOFs are dependent, u_s = T [u_master; joint DOFs], with T
// rebuilt from the current geometry (masterSlaveJointRoutinesModule.f90:
// 374-577, updateDependencies) and the slave placed on its kinematic position
// (:218-299, moveJointInPosition) before every element update.
struct Joint {
  int id = 0, type = 0;
  int slave = -1, master = -1;  // triad indices
  M34 JPosInG, JPosInT, STPos0InJ;
  int nMats = 0;
  std::vector<int> lDof, iMat, BC;  // per joint DOF (iMat 1-based)
  std::vector<double> jVar, jVarPrev;
  int firstDof = -1;  // first joint DOF in the DOF vectors
  int nM = 0;         // master DOFs in the constraint (0 for a grounded master)
  int ncol = 0;       // nM + joint DOFs
  double TR[3][3];
  std::vector<double> T;      // 6 x ncol, row-major
  std::vector<int> colEq;     // 0-based equation of each column, -1 fixed/prescribed
};

struct TestItem {
  int code = -1;  // 1 allOf, 2 oneOf, -1 inactive
  double absTol = 0.0, value = 0.0;
};

}  // namespace

struct OracleModel {
  Options opt;
  std::vector<Triad> triads;
  std::vector<Prop> props;
  std::vector<Elem> elems;
  std::vector<Load> loads;
  std::vector<Func> funcs;
  std::vector<Sensor> sensors;
  std::vector<EngineF> engines;
  std::vector<Motion> motions;
  std::vector<Axial> axials;    // springs first, then dampers (assembly order)
  std::vector<Joint> joints;
  std::vector<int> dep;         // per DOF: 6 * joint + row of a dependent DOF, else -1
  std::vector<int> axEq;        // 6 per axial element: 0-based equation, -1 fixed, <= -2 prescribed
  const std::vector<double>* axVel = nullptr;  // triad velocities the dampers see
  std::vector<double> ccv;  // constant term of each constraint equation (TTCC(MPMCEQ(iceq)))
  double tQStatic = -1.0e99;  // end of the quasi-static load steps
  int quasiSteps = 0;         // quasi-static steps since the last dynamic one
  std::vector<double> urdp, urddp;
  double gravity[3] = {0, 0, 0};
  double wDisp[3] = {1, 1, 1}, wForce[3] = {1, 1, 1};

  // SAM
  int ndof = 0, neq = 0;
  std::vector<int> meqn, dofType;
  std::vector<int> elEq;   // n per element: 0-based equation, -1 fixed, <= -2 prescribed
  std::vector<int> elOff;  // start of each element's codes in elEq

  // skyline (upper profile, column oriented)
  std::vector<int> first;      // first row of each column
  std::vector<long> colptr;    // start of column storage; diag at colptr[j] + j - first[j]
  std::vector<double> sky;

  // CSR upper pattern (parity)
  std::vector<int> rowptr, cols;

  // time integration state (SystemType, systemTypeModule.f90:23-111)
  double alpha = -0.1, beta = 0.3025, gamma = 0.6;
  double time = 0.0, timeStep = 0.0, tStart = 0.0, tEnd = 0.0, tInc = 0.0, minInc = 0.001;
  double sacc = 0.0, svel = 0.0;
  long long nStep = 0, nIter = 0;
  int nIterThisStep = 0, maxIt = 15, minIt = 1, fixedIt = 0, nUpdat = 0, maxSeqNoUpdate = 100;
  double tolUpdateFactor = 0.0;
  int stiffDampFiltering = 1;
  std::vector<double> urd, urdd, dk, ak, rinc, sinc[3];
  std::vector<double> FSk, FDk, FIk, Qk, FIactual, residual, del;
  TestItem dis[4], vel[4], acc[4], res[4], ener[2];
  double lastNorms[4] = {0, 0, 0, 0};
  bool haveMat = false;  // skyline holds a factorization
  double oldScale[3] = {-1, -1, -1};
  bool finished = false;
  int error = 0;
  // largest triad displacement from the start positions seen at the end of any
  // step so far (the scale of the response over the run, for relative errors)
  std::vector<double> x0;
  double maxDisp = 0.0;
};

namespace {

// ---------------------------------------------------------------------------
// Model set-up
// ---------------------------------------------------------------------------

static void rowMajor34(const std::vector<double>& v, M34 T) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) T[r][c] = (size_t)(4 * r + c) < v.size() ? v[4 * r + c] : 0.0;
}

static int findTriad(const OracleModel& m, int id) {
  for (size_t k = 0; k < m.triads.size(); ++k)
    if (m.triads[k].id == id) return (int)k;
  return -1;
}

// Superelement corotated frame (supElTypeModule.f90:912-992, shadowPosAlg = 1).
static int updateCorot(const OracleModel& m, Elem& e, bool init) {
  double pnt[3][3];
  for (int j = 0; j < 3; ++j) {
    const Triad& t = m.triads[e.tri[e.ref[j]]];
    for (int r = 0; r < 3; ++r)
      pnt[j][r] = t.ur[r][0] * e.offset[j][0] + t.ur[r][1] * e.offset[j][1] + t.ur[r][2] * e.offset[j][2] +
                  t.ur[r][3];
  }
  M34 triTr;
  if (trans3P(pnt[0], pnt[1], pnt[2], triTr) != 0) return -1;
  if (init) {
    M34 inv;
    invert34(triTr, inv);
    matmul34(inv, e.supTr, e.triRelSup);
  } else {
    matmul34(triTr, e.triRelSup, e.supTr);
  }
  return 0;
}

// Deformation vector in corotated axes (supElTypeModule.f90:1067-1114).
static void buildFinit(const OracleModel& m, Elem& e) {
  M34 inv;
  invert34(e.supTr, inv);
  for (int i = 0; i < e.nTri; ++i) {
    M34 loc;
    matmul34(inv, m.triads[e.tri[i]].ur, loc);
    double* f = e.finit.data() + 6 * i;
    for (int r = 0; r < 3; ++r) f[r] = loc[r][3] - e.tu(i, r, 3);
    double dR[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)
        dR[r][c] = loc[r][0] * e.tu(i, 0, c) + loc[r][1] * e.tu(i, 1, c) + loc[r][2] * e.tu(i, 2, c);
    f[3] = dR[2][1];
    f[4] = dR[0][2];
    f[5] = dR[1][0];
  }
  // generalized DOFs (:1108-1112)
  for (int g = 0; g < e.nGen; ++g) e.finit[6 * e.nTri + g] = e.genUr[g];
}

// y = s * A x, A n x n column-major (the leading nr rows and columns when nr < n)
static void matvecN(const double* A, int n, const double* x, double s, double* y, int nr = -1) {
  if (nr < 0) nr = n;
  for (int i = 0; i < nr; ++i) {
    double t = 0.0;
    for (int j = 0; j < nr; ++j) t += A[i + (size_t)n * j] * x[j];
    y[i] = s * t;
  }
}

// System DOF (0-based) of local DOF i of an element: triad DOFs, then the
// generalized DOFs (csExtractElv / MADOF order of the element's SAM nodes).
static int elemDof(const OracleModel& m, const Elem& e, int i) {
  return i < 6 * e.nTri ? m.triads[e.tri[i / 6]].firstDof + i % 6 : e.genFirstDof + (i - 6 * e.nTri);
}

// Element velocity/acceleration in corotated axes (supElRoutinesModule.f90:47-85);
// the generalized DOFs are copied.
static void setElemVelAcc(const OracleModel& m, Elem& e, const std::vector<double>& v,
                          const std::vector<double>& a) {
  for (int i = 0; i < e.nTri; ++i) {
    int d = m.triads[e.tri[i]].firstDof;
    for (int g = 0; g < 2; ++g) {
      double vv[3], aa[3];
      for (int r = 0; r < 3; ++r) { vv[r] = v[d + 3 * g + r]; aa[r] = a[d + 3 * g + r]; }
      for (int r = 0; r < 3; ++r) {
        e.uld[6 * i + 3 * g + r] = e.supTr[0][r] * vv[0] + e.supTr[1][r] * vv[1] + e.supTr[2][r] * vv[2];
        e.uldd[6 * i + 3 * g + r] = e.supTr[0][r] * aa[0] + e.supTr[1][r] * aa[1] + e.supTr[2][r] * aa[2];
      }
    }
  }
  for (int g = 0; g < e.nGen; ++g) {
    e.uld[6 * e.nTri + g] = v[e.genFirstDof + g];
    e.uldd[6 * e.nTri + g] = a[e.genFirstDof + g];
  }
}

// triad DOF groups to system directions (UpdateSupEls :410-450); the
// generalized DOFs keep their values
static void rotateOut(const Elem& e, double* f) {
  for (int g = 0; g < 2 * e.nTri; ++g) {
    double x[3] = {f[3 * g], f[3 * g + 1], f[3 * g + 2]};
    for (int r = 0; r < 3; ++r) f[3 * g + r] = e.supTr[r][0] * x[0] + e.supTr[r][1] * x[1] + e.supTr[r][2] * x[2];
  }
}

// spin(v) x = v x x (rotationModule)
static void spinMat(const double* v, double S[3][3]) {
  S[0][0] = 0.0;   S[0][1] = -v[2]; S[0][2] = v[1];
  S[1][0] = v[2];  S[1][1] = 0.0;   S[1][2] = -v[0];
  S[2][0] = -v[1]; S[2][1] = v[0];  S[2][2] = 0.0;
}

// position matrix of the joint variables of level iMat (1-based): translations
// of its translational DOFs and the rotation of its (at most one) rotational DOF
static void jointPosFromVars(const Joint& J, int im, M34 P) {
  double th[3] = {0.0, 0.0, 0.0};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) P[r][c] = 0.0;
  for (size_t k = 0; k < J.lDof.size(); ++k) {
    if (J.iMat[k] != im) continue;
    if (J.lDof[k] <= 3) P[J.lDof[k] - 1][3] = J.jVar[k];
    else th[J.lDof[k] - 4] = J.jVar[k];
  }
  double R[3][3];
  vec_to_mat(th, R);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) P[r][c] = R[r][c];
}

// moveJointInPosition (masterSlaveJointRoutinesModule.f90:218-299, one master
// triad) followed by updateDependencies (:374-577) for a joint whose dependent
// triad has global system directions and no prescribed master or joint DOFs
static void updateJoint(OracleModel& m, Joint& J) {
  Triad& S = m.triads[J.slave];
  const Triad& Mt = m.triads[J.master];
  matmul34(Mt.ur, J.JPosInT, J.JPosInG);
  double e[3];
  for (int k = 0; k < 3; ++k) e[k] = -(S.ur[k][3] - Mt.ur[k][3]);
  spinMat(e, J.TR);  // TR = -spin(e), e = dependent triad relative to the master
  M34 P, Q;
  std::memcpy(P, J.STPos0InJ, sizeof(M34));
  for (int i = 1; i <= J.nMats; ++i) {
    M34 F;
    jointPosFromVars(J, i, F);
    matmul34(F, P, Q);
    std::memcpy(P, Q, sizeof(M34));
  }
  matmul34(J.JPosInG, P, S.ur);
  // constraint coefficients
  std::fill(J.T.begin(), J.T.end(), 0.0);
  const int nc = J.ncol;
  for (int lm = 0; lm < J.nM; ++lm)
    for (int ls = 0; ls < 6; ++ls) {
      double v = 0.0;
      if (ls < 3 && lm < 3) v = ls == lm ? 1.0 : 0.0;
      else if (ls < 3) v = J.TR[ls][lm - 3];
      else if (lm >= 3) v = ls == lm ? 1.0 : 0.0;
      J.T[ls * nc + lm] = v;
    }
  std::vector<M34> csys(J.nMats + 1), png(J.nMats + 1);
  M34 Pacc;
  std::memcpy(Pacc, J.JPosInG, sizeof(M34));
  for (int i = J.nMats; i >= 1; --i) {
    std::memcpy(csys[i], Pacc, sizeof(M34));
    M34 F, N;
    jointPosFromVars(J, i, F);
    matmul34(Pacc, F, N);
    std::memcpy(Pacc, N, sizeof(M34));
    std::memcpy(png[i], Pacc, sizeof(M34));
  }
  for (size_t k = 0; k < J.lDof.size(); ++k) {
    const int lm = J.lDof[k], im = J.iMat[k];
    double dUS[6];
    if (lm <= 3) {
      for (int r = 0; r < 3; ++r) { dUS[r] = csys[im][r][lm - 1]; dUS[3 + r] = 0.0; }
    } else {
      double dOm[3], ecc[3], dUG[3];
      for (int r = 0; r < 3; ++r) {
        dOm[r] = csys[im][r][lm - 4];
        ecc[r] = S.ur[r][3] - png[im][r][3];
      }
      cross(dOm, ecc, dUG);
      for (int r = 0; r < 3; ++r) { dUS[r] = dUG[r]; dUS[3 + r] = dOm[r]; }
    }
    for (int ls = 0; ls < 6; ++ls) J.T[ls * nc + J.nM + (int)k] = dUS[ls];
  }
}

static void updateJoints(OracleModel& m) {
  for (Joint& J : m.joints) updateJoint(m, J);
}

// IncJointsVar (masterSlaveJointRoutinesModule.f90:40-99): joint variables += increments
static void incJointsVar(OracleModel& m, const std::vector<double>& inc) {
  for (Joint& J : m.joints)
    for (size_t k = 0; k < J.jVar.size(); ++k) J.jVar[k] += inc[J.firstDof + k];
}

struct Term {
  int eq;
  double c;
};

// equations and coefficients a DOF's value contributes to (MEEN < 0 expands
// through MPMCEQ/MMCEQ/TTCC, sysMatrixTypeModule.f90:2099-2259)
static void dofTerms(const OracleModel& m, int d, std::vector<Term>& out) {
  out.clear();
  if (m.dep[d] >= 0) {
    const Joint& J = m.joints[m.dep[d] / 6];
    const int r = m.dep[d] % 6;
    for (int c = 0; c < J.ncol; ++c)
      if (J.colEq[c] >= 0) out.push_back({J.colEq[c], J.T[r * J.ncol + c]});
  } else if (m.meqn[d] > 0) {
    out.push_back({m.meqn[d] - 1, 1.0});
  }
}

static bool elemConstrained(const OracleModel& m, const Elem& e) {
  for (int i = 0; i < e.nTri; ++i)
    if (m.dep[m.triads[e.tri[i]].firstDof] >= 0) return true;
  return false;
}

// Element forces (supElRoutinesModule.f90:231-456, UpdateSupEls; and :460-630,
// UpdateSupElsStatic when isStatic).  The joints are updated first, as
// UpdateMechanism does (newmarkRoutinesModule.f90:206-323).
static int updateElems(OracleModel& m, bool newPositions, bool isStatic, bool corotInStatic) {
  updateJoints(m);
  for (Elem& e : m.elems) {
    if (newPositions || (isStatic && corotInStatic)) {
      if (updateCorot(m, e, false) != 0) return -1;
      buildFinit(m, e);
    } else if (isStatic) {
      buildFinit(m, e);
    }
    const int n = e.n;
    if (isStatic) {
      for (int k = 0; k < n; ++k) { e.FI[k] = 0.0; e.FD[k] = 0.0; }
    } else {
      matvecN(e.M.data(), n, e.uldd.data(), 1.0, e.FI.data());
      if (e.hasC)
        matvecN(e.C.data(), n, e.uld.data(), e.stifScl, e.FD.data());
      else
        for (int k = 0; k < n; ++k) e.FD[k] = 0.0;
      if (m.timeStep > 0.0 && e.hasVld) {
        // rigid-body filtering of the stiffness-proportional damping on the
        // triad DOFs: Fd -= alpha2 K (uld - vld), vld = (finit - finitPrev) / h
        const int nv = 6 * e.nTri;
        std::vector<double> tmp(nv), fs(nv);
        for (int k = 0; k < nv; ++k) e.vld[k] = (e.finit[k] - e.finitPrev[k]) / m.timeStep;
        for (int k = 0; k < nv; ++k) tmp[k] = e.uld[k] - e.vld[k];
        matvecN(e.K.data(), n, tmp.data(), e.stifScl, fs.data(), nv);
        for (int k = 0; k < nv; ++k) e.FD[k] -= e.kDmp * fs[k];
      }
    }
    matvecN(e.K.data(), n, e.finit.data(), e.stifScl, e.FS.data());
    double gl[3];
    for (int c = 0; c < 3; ++c)
      gl[c] = m.gravity[0] * e.supTr[0][c] + m.gravity[1] * e.supTr[1][c] + m.gravity[2] * e.supTr[2][c];
    for (int i = 0; i < n; ++i)
      e.Q[i] = e.stifScl * (e.fg[i] * gl[0] + e.fg[i + n] * gl[1] + e.fg[i + 2 * n] * gl[2]);
    rotateOut(e, e.FS.data());
    rotateOut(e, e.Q.data());
    if (!isStatic) {
      rotateOut(e, e.FD.data());
      rotateOut(e, e.FI.data());
    }
  }
  // axial springs and dampers (UpdateSprings / UpdateDampers, then
  // calcSpringForces / addInDampingForces / calcDamperForces)
  for (Axial& a : m.axials) {
    const Triad& t1 = m.triads[a.tri[0]];
    const Triad& t2 = m.triads[a.tri[1]];
    double d[3] = {t2.ur[0][3] - t1.ur[0][3], t2.ur[1][3] - t1.ur[1][3], t2.ur[2][3] - t1.ur[2][3]};
    double l2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (l2 < epsDiv0) {
      if (a.kind == 0) return -1;  // the two points defining the spring coincide
      a.L = std::sqrt(l2);
      a.n[0] = a.n[1] = a.n[2] = 0.0;
    } else {
      a.L = std::sqrt(l2);
      for (int k = 0; k < 3; ++k) a.n[k] = d[k] / a.L;
    }
    double v1[3] = {0, 0, 0}, v2[3] = {0, 0, 0};
    if (!isStatic && m.axVel) {
      for (int k = 0; k < 3; ++k) {
        v1[k] = (*m.axVel)[t1.firstDof + k];
        v2[k] = (*m.axVel)[t2.firstDof + k];
      }
    }
    for (int k = 0; k < 6; ++k) a.FS[k] = a.FD[k] = 0.0;
    if (a.kind == 0) {
      a.F = a.s0 * (a.L - a.l0);
      for (int k = 0; k < 3; ++k) {
        a.FS[k] = 0.0 - a.F * a.n[k];
        a.FS[3 + k] = 0.0 + a.F * a.n[k];
      }
      if (!isStatic && std::fabs(a.alpha2) > 1.0e-16) {
        // stiffness-proportional damping forces C v with C = alpha2 * s0 * n n^T blocks
        double km = a.s0 * a.alpha2 * a.L / a.L;
        for (int i = 0; i < 3; ++i) {
          double f1 = 0.0, f2 = 0.0;
          for (int j = 0; j < 3; ++j) f1 += a.n[i] * a.n[j] * km * v1[j];
          for (int j = 0; j < 3; ++j) f1 += -(a.n[i] * a.n[j] * km) * v2[j];
          for (int j = 0; j < 3; ++j) f2 += -(a.n[i] * a.n[j] * km) * v1[j];
          for (int j = 0; j < 3; ++j) f2 += a.n[i] * a.n[j] * km * v2[j];
          a.FD[i] = f1;
          a.FD[3 + i] = f2;
        }
      }
    } else {
      double vr[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
      double vel = a.n[0] * vr[0] + a.n[1] * vr[1] + a.n[2] * vr[2];
      a.F = a.d0 * vel;
      if (!isStatic)
        for (int k = 0; k < 3; ++k) {
          a.FD[k] = -a.F * a.n[k];
          a.FD[3 + k] = -a.FD[k];
        }
    }
  }
  return 0;
}

// 3x3 translational block of an axial element's Newton matrix
// (calcSpringStiffness without geometric stiffness; addInDamperMat)
static void axialBlock(const Axial& a, double sC, double sK, double* A) {
  if (a.kind == 0) {
    const double km = (a.s0 * (sK + sC * a.alpha2)) * a.L / a.L;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) A[i + 3 * j] = a.n[i] * a.n[j] * km;
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) A[i + 3 * j] = a.n[i] * a.n[j] * a.d0 * sC;
  }
}

// System force vectors (addInSysModule.f90:626-840, GetForceVectors).
static void getForceVectors(OracleModel& m) {
  std::fill(m.FSk.begin(), m.FSk.end(), 0.0);
  std::fill(m.FDk.begin(), m.FDk.end(), 0.0);
  std::fill(m.FIk.begin(), m.FIk.end(), 0.0);
  std::fill(m.Qk.begin(), m.Qk.end(), 0.0);
  std::vector<Term> terms;
  for (size_t k = 0; k < m.elems.size(); ++k) {
    const Elem& e = m.elems[k];
    const int* eq = &m.elEq[m.elOff[k]];
    if (elemConstrained(m, e)) {
      // csAddEV through the constraint equations of dependent DOFs
      for (int i = 0; i < e.n; ++i) {
        dofTerms(m, elemDof(m, e, i), terms);
        for (const Term& t : terms) {
          m.FSk[t.eq] += t.c * e.FS[i];
          m.FDk[t.eq] += t.c * e.FD[i];
          m.FIk[t.eq] += t.c * e.FI[i];
          m.Qk[t.eq] += t.c * e.Q[i];
        }
      }
      continue;
    }
    for (int i = 0; i < e.n; ++i) {
      if (eq[i] < 0) continue;
      m.FSk[eq[i]] += e.FS[i];
      m.FDk[eq[i]] += e.FD[i];
      m.FIk[eq[i]] += e.FI[i];
      m.Qk[eq[i]] += e.Q[i];
    }
  }
  for (size_t k = 0; k < m.axials.size(); ++k) {
    const Axial& a = m.axials[k];
    const int* eq = &m.axEq[6 * k];
    for (int i = 0; i < 6; ++i) {
      if (eq[i] < 0) continue;
      m.FSk[eq[i]] += a.FS[i];
      m.FDk[eq[i]] += a.FD[i];
    }
  }
  for (Load& l : m.loads) {
    const Triad& t = m.triads[l.triad];
    int d = t.firstDof + l.dof - 1;
    int eq = m.meqn[d] - 1;
    if (eq >= 0) m.Qk[eq] += l.F;
  }
}

// Engine value at the current time (engineRoutinesModule.f90:163-240 subset).
static double engineValue(const OracleModel& m, int e) {
  const EngineF& en = m.engines[e];
  double x = m.time;  // TIME sensor (or no sensor)
  if (en.sensor >= 0 && lower(m.sensors[en.sensor].type) != "time") x = 0.0;
  if (en.func < 0) return x;
  const Func& f = m.funcs[en.func];
  std::string t = lower(f.type);
  if (t == "scale") return (f.real.empty() ? 1.0 : f.real[0]) * x;
  if (t == "constant") return f.real.empty() ? 0.0 : f.real[0];
  if (t == "sinusoidal") {  // realData: frequency, delay (periods), amplitude, mean
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t k = 0; k < 4 && k < f.real.size(); ++k) p[k] = f.real[k];
    return p[3] + p[2] * std::sin(2.0 * M_PI * (p[0] * x - p[1]));
  }
  return x;
}

// External load values F = f0 + f1 * engine (forceRoutinesModule.f90:52-131, Evaluate).
static void updateLoads(OracleModel& m) {
  for (Load& l : m.loads) l.F = l.engine >= 0 ? l.f0 + l.f1 * engineValue(m, l.engine) : l.f0;
}

// Prescribed motions (motionRoutinesModule.f90:58-193): D = d0 + d1 * engine;
// the constraint constant is the total value in linear statics, else the increment.
static void updatePrescribedMotions(OracleModel& m, bool linearStatic) {
  for (Motion& mo : m.motions) {
    double Dprev = mo.D;
    mo.D = mo.engine >= 0 ? mo.d0 + mo.d1 * engineValue(m, mo.engine) : mo.d0;
    m.ccv[mo.iceq - 1] = linearStatic ? mo.D : mo.D - Dprev;
  }
}

// ---------------------------------------------------------------------------
// Skyline LDL^T
// ---------------------------------------------------------------------------

static void skylineClear(OracleModel& m) { std::fill(m.sky.begin(), m.sky.end(), 0.0); }

static inline double& skyAt(OracleModel& m, int i, int j) {  // i <= j
  return m.sky[m.colptr[j] + (i - m.first[j])];
}

// Newton matrix N = sM*M + sC*C + sK*K, rotated to system axes and added to
// the upper triangle (supElRoutinesModule.f90:1127-1187 AddInSupMat + MATTRA;
// sysMatrixTypeModule.f90:2099-2259 asmSparse semantics for free DOFs).
static void rotatedElementMatrix(const Elem& e, const double* Nloc, double* Ns) {
  // Ns = R * N * R^T on the triad DOF groups, R = supTr(:,1:3); the rows and
  // columns of generalized DOFs are not rotated (MATTRA on the triad groups only)
  const int n = e.n, nb = 2 * e.nTri, nt = 6 * e.nTri;
  for (int bi = 0; bi < nb; ++bi)
    for (int bj = 0; bj < nb; ++bj) {
      double B[3][3], W[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) B[r][c] = Nloc[(3 * bi + r) + (size_t)n * (3 * bj + c)];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) W[r][c] = e.supTr[r][0] * B[0][c] + e.supTr[r][1] * B[1][c] + e.supTr[r][2] * B[2][c];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          Ns[(3 * bi + r) + (size_t)n * (3 * bj + c)] =
              W[r][0] * e.supTr[c][0] + W[r][1] * e.supTr[c][1] + W[r][2] * e.supTr[c][2];
    }
  for (int bi = 0; bi < nb; ++bi)
    for (int j = nt; j < n; ++j) {
      const double* b = Nloc + 3 * bi + (size_t)n * j;
      for (int r = 0; r < 3; ++r)
        Ns[(3 * bi + r) + (size_t)n * j] = e.supTr[r][0] * b[0] + e.supTr[r][1] * b[1] + e.supTr[r][2] * b[2];
    }
  for (int i = nt; i < n; ++i)
    for (int bj = 0; bj < nb; ++bj) {
      double b[3];
      for (int c = 0; c < 3; ++c) b[c] = Nloc[i + (size_t)n * (3 * bj + c)];
      for (int c = 0; c < 3; ++c)
        Ns[i + (size_t)n * (3 * bj + c)] = b[0] * e.supTr[c][0] + b[1] * e.supTr[c][1] + b[2] * e.supTr[c][2];
    }
  for (int i = nt; i < n; ++i)
    for (int j = nt; j < n; ++j) Ns[i + (size_t)n * j] = Nloc[i + (size_t)n * j];
}

static void buildElementNewton(Elem& e, double sM, double sC, double sK) {
  // supElRoutinesModule.f90:1254-1320, BuildSupNewtonMat (material stiffness)
  for (int k = 0; k < e.n * e.n; ++k) {
    double v = sM * e.M[k];
    if (e.hasC) v += sC * e.stifScl * e.C[k];
    v += sK * e.stifScl * e.K[k];
    e.N[k] = v;
  }
}

// Element equation codes: >= 0 equation, -1 fixed, <= -2 prescribed DOF of
// constraint equation iceq = -1 - code (asmSparse, sysMatrixTypeModule.f90:2099-2259:
// rows/columns of constrained DOFs leave the matrix; with a right-hand side the
// constant term c moves as B(jeq) -= c * EM(i,j)).
static void assembleSkyline(OracleModel& m, double sM, double sC, double sK, std::vector<double>* rhs = nullptr) {
  skylineClear(m);
  bool rebuild = std::fabs(sM - m.oldScale[0]) + std::fabs(sK - m.oldScale[1]) + std::fabs(sC - m.oldScale[2]) > 1.0e-16;
  if (rebuild) {
    m.oldScale[0] = sM; m.oldScale[1] = sK; m.oldScale[2] = sC;
    for (Elem& e : m.elems) buildElementNewton(e, sM, sC, sK);
  }
  std::vector<double> NsV;
  std::vector<Term> ti, tj;
  for (size_t k = 0; k < m.elems.size(); ++k) {
    const Elem& e = m.elems[k];
    const int n = e.n;
    NsV.resize((size_t)n * n);
    double* Ns = NsV.data();
    rotatedElementMatrix(e, e.N.data(), Ns);
    const int* eq = &m.elEq[m.elOff[k]];
    if (elemConstrained(m, e)) {
      // T^T N T: every pair of terms, upper triangle (asmSparse with MEEN < 0)
      for (int i = 0; i < n; ++i) {
        dofTerms(m, elemDof(m, e, i), ti);
        for (int j = 0; j < n; ++j) {
          dofTerms(m, elemDof(m, e, j), tj);
          for (const Term& a : ti)
            for (const Term& b : tj)
              if (b.eq >= a.eq) skyAt(m, a.eq, b.eq) += a.c * b.c * Ns[i + (size_t)n * j];
        }
      }
      continue;
    }
    for (int i = 0; i < n; ++i) {
      if (eq[i] < 0) continue;
      for (int j = 0; j < n; ++j) {
        if (eq[j] < eq[i]) continue;
        skyAt(m, eq[i], eq[j]) += Ns[i + (size_t)n * j];
      }
    }
    if (!rhs) continue;
    for (int i = 0; i < n; ++i) {
      if (eq[i] > -2) continue;
      double c = m.ccv[-2 - eq[i]];
      if (!(std::fabs(c) > 1.0e-15)) continue;
      for (int j = 0; j < n; ++j)
        if (eq[j] >= 0) (*rhs)[eq[j]] -= c * Ns[i + (size_t)n * j];
    }
  }
  for (size_t k = 0; k < m.axials.size(); ++k) {
    double A[9], E[36];
    axialBlock(m.axials[k], sC, sK, A);
    for (int bj = 0; bj < 2; ++bj)
      for (int bi = 0; bi < 2; ++bi)
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) E[(3 * bi + r) + 6 * (3 * bj + c)] = bi == bj ? A[r + 3 * c] : -A[r + 3 * c];
    const int* eq = &m.axEq[6 * k];
    for (int i = 0; i < 6; ++i) {
      if (eq[i] < 0) continue;
      for (int j = 0; j < 6; ++j) {
        if (eq[j] < eq[i]) continue;
        skyAt(m, eq[i], eq[j]) += E[i + 6 * j];
      }
    }
    if (!rhs) continue;
    for (int i = 0; i < 6; ++i) {
      if (eq[i] > -2) continue;
      double c = m.ccv[-2 - eq[i]];
      if (!(std::fabs(c) > 1.0e-15)) continue;
      for (int j = 0; j < 6; ++j)
        if (eq[j] >= 0) (*rhs)[eq[j]] -= c * E[i + 6 * j];
    }
  }
}

// Profile LDL^T; returns -3 on a singular pivot, else the number of negative pivots.
static int skylineFactor(OracleModel& m, double tol) {
  int n = m.neq, nneg = 0;
  for (int j = 0; j < n; ++j) {
    int fj = m.first[j];
    double* cj = &m.sky[m.colptr[j]] - fj;  // cj[i] = entry (i,j)
    double ajj = cj[j];
    for (int i = fj + 1; i < j; ++i) {
      int fi = m.first[i];
      const double* ci = &m.sky[m.colptr[i]] - fi;
      int k0 = std::max(fi, fj);
      double s = 0.0;
      for (int k = k0; k < i; ++k) s += ci[k] * cj[k];
      cj[i] -= s;
    }
    double d = ajj;
    for (int i = fj; i < j; ++i) {
      double g = cj[i];
      double l = g / m.sky[m.colptr[i] + (i - m.first[i])];
      cj[i] = l;
      d -= l * g;
    }
    if (std::fabs(d) <= tol * std::fabs(ajj) || d == 0.0) return -3;
    if (d < 0.0) ++nneg;
    cj[j] = d;
  }
  return nneg;
}

static void skylineSolve(const OracleModel& m, std::vector<double>& b) {
  int n = m.neq;
  for (int j = 0; j < n; ++j) {
    int fj = m.first[j];
    const double* cj = &m.sky[m.colptr[j]] - fj;
    double s = 0.0;
    for (int i = fj; i < j; ++i) s += cj[i] * b[i];
    b[j] -= s;
  }
  for (int j = 0; j < n; ++j) b[j] /= m.sky[m.colptr[j] + (j - m.first[j])];
  for (int j = n - 1; j >= 0; --j) {
    int fj = m.first[j];
    const double* cj = &m.sky[m.colptr[j]] - fj;
    double x = b[j];
    for (int i = fj; i < j; ++i) b[i] -= cj[i] * x;
  }
}

// ---------------------------------------------------------------------------
// Norms (normRoutinesModule.f90:83-340, solverRoutinesModule.f90:285-380)
// ---------------------------------------------------------------------------

// Equation order -> DOF order (csExpand, solExtensionModule.f90:1352-1387):
// free DOFs take the solution, prescribed DOFs F2 times their constant term.
static void expandEq(const OracleModel& m, const std::vector<double>& eqv, std::vector<double>& dofv,
                     double F2 = 1.0) {
  dofv.assign(m.ndof, 0.0);
  for (int d = 0; d < m.ndof; ++d) {
    if (m.meqn[d] > 0) dofv[d] = eqv[m.meqn[d] - 1];
    else if (m.meqn[d] < 0) dofv[d] = F2 * m.ccv[-m.meqn[d] - 1];
    else if (m.dep[d] >= 0) {  // dependent DOF: its constraint equation (constant term 0)
      const Joint& J = m.joints[m.dep[d] / 6];
      const int r = m.dep[d] % 6;
      double v = 0.0;
      for (int c = 0; c < J.ncol; ++c)
        if (J.colEq[c] >= 0) v += J.T[r * J.ncol + c] * eqv[J.colEq[c]];
      dofv[d] = v;
    }
  }
}

static double scaledNorm(const OracleModel& m, const std::vector<double>& v, const double* w) {
  double sw = 0.0, rn = 0.0;
  for (int d = 0; d < m.ndof; ++d) {
    if (m.meqn[d] <= 0) continue;
    double wf = w[m.dofType[d] - 1];
    sw += wf * wf;
    rn += (wf * v[d]) * (wf * v[d]);
  }
  return sw > 0.0 ? std::sqrt(rn / sw) : 0.0;
}

static void infNorms(const OracleModel& m, const std::vector<double>& v, double* out3) {
  out3[0] = out3[1] = out3[2] = 0.0;
  for (int d = 0; d < m.ndof; ++d) {
    if (m.meqn[d] <= 0) continue;
    double a = std::fabs(v[d]);
    int t = m.dofType[d] - 1;
    if (a > out3[t]) out3[t] = a;
  }
}

static void calculateNorms(OracleModel& m) {
  std::vector<double> resx;
  expandEq(m, m.residual, resx);
  m.dis[0].value = scaledNorm(m, m.sinc[0], m.wDisp);
  m.vel[0].value = scaledNorm(m, m.sinc[1], m.wDisp);
  m.acc[0].value = scaledNorm(m, m.sinc[2], m.wDisp);
  m.res[0].value = scaledNorm(m, resx, m.wForce);
  double t3[3];
  infNorms(m, m.sinc[0], t3);
  for (int k = 0; k < 3; ++k) m.dis[k + 1].value = t3[k];
  infNorms(m, m.sinc[1], t3);
  for (int k = 0; k < 3; ++k) m.vel[k + 1].value = t3[k];
  infNorms(m, m.sinc[2], t3);
  for (int k = 0; k < 3; ++k) m.acc[k + 1].value = t3[k];
  infNorms(m, resx, t3);
  for (int k = 0; k < 3; ++k) m.res[k + 1].value = t3[k];
  double esum = 0.0, emax = 0.0;
  for (int d = 0; d < m.ndof; ++d) {
    if (m.meqn[d] <= 0) continue;
    double e = std::fabs(m.sinc[0][d] * resx[d]);
    esum += e;
    if (e > emax) emax = e;
  }
  if (m.ndof > 1 && m.neq > 0) esum /= (double)m.neq;
  m.ener[0].value = emax;
  m.ener[1].value = esum;
  m.lastNorms[0] = m.dis[0].value;
  m.lastNorms[1] = m.vel[0].value;
  m.lastNorms[2] = m.acc[0].value;
  m.lastNorms[3] = m.res[0].value;
}

// normTypeModule.f90:196-249, HasConverged
static bool hasConverged(const OracleModel& m) {
  bool exists[3] = {false, false, false}, oneOf = false, allOf = true;
  auto test = [&](const TestItem& t) {
    if (t.code == 2) { if (t.value < t.absTol) oneOf = true; }
    else if (t.code == 1) { if (t.value >= t.absTol) allOf = false; }
    else return;
    exists[t.code] = true;
  };
  for (int k = 0; k < 4; ++k) { test(m.dis[k]); test(m.vel[k]); test(m.acc[k]); test(m.res[k]); }
  test(m.ener[0]);
  test(m.ener[1]);
  bool c = true;
  if (exists[2]) c = c && oneOf;
  if (exists[1]) c = c && allOf;
  return c;
}

static void initTol(const Options& o, const char* key, TestItem& t) {
  double v = o.d(key, 0.0);
  t.value = 0.0;
  if (v > 0.0) { t.absTol = v; t.code = 1; }
  else if (v < 0.0) { t.absTol = -v; t.code = 2; }
  else { t.absTol = 0.0; t.code = -1; }
}

// ---------------------------------------------------------------------------
// Increments (newmarkRoutinesModule.f90:160-187, :418-486; triadTypeModule.f90:677-722)
// ---------------------------------------------------------------------------

static void incTriadsPos(OracleModel& m, const std::vector<double>& inc) {
  for (Triad& t : m.triads) {
    if (t.nDOFs == 0) continue;
    int j = t.firstDof;
    for (int r = 0; r < 3; ++r) t.ur[r][3] += inc[j + r];
    if (t.nDOFs == 6) {
      double R[3][3], U[3][3];
      vec_to_mat(&inc[j + 3], R);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) U[r][c] = R[r][0] * t.ur[0][c] + R[r][1] * t.ur[1][c] + R[r][2] * t.ur[2][c];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t.ur[r][c] = U[r][c];
    }
  }
}

// IncSupElsGenDofs (supElRoutinesModule.f90:168-200): generalized DOFs += increments
static void incGenDofs(OracleModel& m, const std::vector<double>& inc) {
  for (Elem& e : m.elems)
    for (int g = 0; g < e.nGen; ++g) e.genUr[g] += inc[e.genFirstDof + g];
}

static void incAll(OracleModel& m, const std::vector<double>& inc) {
  incTriadsPos(m, inc);
  incGenDofs(m, inc);
  incJointsVar(m, inc);
}

static int factorNewton(OracleModel& m, double sM, double sC, double sK) {
  assembleSkyline(m, sM, sC, sK);
  int ierr = skylineFactor(m, 1.0e-12);
  return ierr;
}

// ---------------------------------------------------------------------------
// Initial static equilibrium (staticEquilibriumModule.f90:50-437)
// ---------------------------------------------------------------------------

static int staticEquilibrium(OracleModel& m) {
  bool initEq = m.opt.b("initEquilibrium", false);
  double equTol = initEq ? m.opt.d("tolInitEquil", 1.0e-3) : 0.0;
  double equLim = initEq ? m.opt.d("limInitEquilStep", 1.0) : 0.0;
  int doIter = 0;
  if (equLim > 0.0 && m.neq > 0) doIter = equTol > 0.0 ? 2 : 1;
  // staticIncAndUpdate without increment: linInc = 1, finit from the initial frame
  std::fill(m.rinc.begin(), m.rinc.end(), 0.0);
  if (updateElems(m, false, true, false) != 0) return -1;
  if (doIter > 0) {
    m.nIterThisStep = 0;
    bool converged = false;
    for (int ninc = 0; ninc < m.maxIt && !converged; ++ninc) {
      bool restart = false;
      for (int it = 1; it <= m.maxIt; ++it) {
        getForceVectors(m);
        for (int k = 0; k < m.neq; ++k) m.residual[k] = m.Qk[k] - m.FSk[k];
        m.del = m.residual;
        assembleSkyline(m, 0.0, 0.0, 1.0);
        int ierr = skylineFactor(m, 1.0e-12);
        if (ierr < 0) return ierr;
        skylineSolve(m, m.del);
        std::vector<double> dx;
        expandEq(m, m.del, dx);
        double deln = scaledNorm(m, dx, m.wDisp);
        if (doIter == 2 && deln > equLim) {
          double f = equLim / deln;
          for (double& v : m.del) v *= f;
        }
        expandEq(m, m.del, m.sinc[0]);
        for (int d = 0; d < m.ndof; ++d) m.rinc[d] += m.sinc[0][d];
        incAll(m, m.sinc[0]);
        if (updateElems(m, false, true, true) != 0) return -1;
        m.nIterThisStep++;
        m.nIter++;
        if (doIter == 1) { converged = true; break; }
        if (deln < equTol && it >= m.minIt) { converged = true; break; }
        if (deln > equLim) { restart = true; break; }
      }
      if (!restart) break;  // not fully converged but accepted
    }
  }
  // finalStaticUpdate (staticEquilibriumModule.f90:1079-1216): zero velocities
  std::fill(m.urd.begin(), m.urd.end(), 0.0);
  std::fill(m.urdd.begin(), m.urdd.end(), 0.0);
  for (Elem& e : m.elems) setElemVelAcc(m, e, m.urd, m.urdd);
  m.axVel = &m.urd;
  double ts = m.timeStep;
  m.timeStep = 0.0;
  updateElems(m, true, false, false);
  m.timeStep = ts;
  for (Triad& t : m.triads) std::memcpy(t.urPrev, t.ur, sizeof(M34));
  for (Elem& e : m.elems) {
    std::memcpy(e.supTrPrev, e.supTr, sizeof(M34));
    e.finitPrev = e.finit;
    e.genUrPrev = e.genUr;
  }
  for (Joint& J : m.joints) J.jVarPrev = J.jVar;
  return 0;
}

// ---------------------------------------------------------------------------
// One time step (newmarkRoutinesModule.f90:551-1118, NewmarkInt, iop = 0,
// NewmarkFlag = 0: HHT-alpha with the eq. (7.53)/(7.55) force predictor/corrector)
// ---------------------------------------------------------------------------

static int newmarkInt(OracleModel& m) {
  m.FIactual = m.FIk;
  m.time += m.timeStep;
  updateLoads(m);
  updatePrescribedMotions(m, false);
  // PredictVelAcc (:85-144)
  double DD = m.gamma / m.beta - 1.0, AA = 0.5 / m.beta - 1.0;
  double DA = (0.5 * m.gamma / m.beta - 1.0) * m.timeStep, AD = 1.0 / (m.beta * m.timeStep);
  for (int d = 0; d < m.ndof; ++d) {
    m.dk[d] = DD * m.urd[d] + DA * m.urdd[d];
    m.ak[d] = AD * m.urd[d] + AA * m.urdd[d];
    m.rinc[d] = 0.0;
  }
  m.sacc = 1.0 / (m.beta * m.timeStep * m.timeStep);
  m.svel = m.gamma / (m.beta * m.timeStep);
  m.nIterThisStep = 0;
  int nSeqNoUpdates = 0;
  double SSTIF = m.alpha + 1.0, SDAMP = m.svel * SSTIF, SMASS = m.sacc;
  for (;;) {
    if (m.nIterThisStep == 0) {
      for (Elem& e : m.elems) setElemVelAcc(m, e, m.dk, m.ak);
      m.axVel = &m.dk;  // SetTriadsVelAcc(triads, dk, ak) in PredictAndUpdate
      if (updateElems(m, false, false, false) != 0) return -1;
      getForceVectors(m);
      for (int k = 0; k < m.neq; ++k)
        m.residual[k] = SSTIF * (m.Qk[k] - m.FSk[k] + m.FDk[k]) + m.FIk[k] - m.alpha * m.FIactual[k];
    } else {
      getForceVectors(m);
      for (int k = 0; k < m.neq; ++k)
        m.residual[k] = SSTIF * (m.Qk[k] - m.FSk[k] - m.FDk[k]) - m.FIk[k] - m.alpha * m.FIactual[k];
    }
    m.del = m.residual;
    bool doTangent;
    if (m.nIterThisStep < std::max(1, m.nUpdat)) doTangent = true;
    else if (nSeqNoUpdates >= m.maxSeqNoUpdate) doTangent = true;
    else doTangent = false;  // tolUpdateFactor <= 1 (default)
    if (doTangent) {
      // the predictor also moves the prescribed-motion terms to the right-hand side
      bool rhsMotion = m.nIterThisStep == 0 && !m.motions.empty();
      assembleSkyline(m, SMASS, SDAMP, SSTIF, rhsMotion ? &m.del : nullptr);
      int ierr = skylineFactor(m, 1.0e-12);
      if (ierr < 0) return ierr;
      nSeqNoUpdates = 0;
    } else {
      ++nSeqNoUpdates;
    }
    skylineSolve(m, m.del);
    // IncAndUpdate: corrector steps replace the prescribed values by zero
    expandEq(m, m.del, m.sinc[0], m.nIterThisStep == 0 ? 1.0 : 0.0);
    for (int d = 0; d < m.ndof; ++d) {
      m.sinc[1][d] = m.sinc[0][d] * m.svel;
      m.sinc[2][d] = m.sinc[0][d] * m.sacc;
      m.rinc[d] += m.sinc[0][d];
      m.urd[d] = m.svel * m.rinc[d] - m.dk[d];
      m.urdd[d] = m.sacc * m.rinc[d] - m.ak[d];
    }
    incAll(m, m.sinc[0]);
    for (Elem& e : m.elems) setElemVelAcc(m, e, m.urd, m.urdd);
    m.axVel = &m.urd;
    if (updateElems(m, true, false, false) != 0) return -1;
    calculateNorms(m);
    m.nIterThisStep++;
    m.nIter++;
    if (m.fixedIt > 0) {
      if (m.nIterThisStep == m.fixedIt) break;
    } else if (m.nIterThisStep > m.maxIt) {
      return 1;  // max iterations without convergence: abort
    } else if (m.nIterThisStep >= std::max(2, m.minIt)) {
      if (hasConverged(m)) break;
    }
  }
  getForceVectors(m);
  return 0;
}

// restoreLastStep (solverRoutinesModule.f90:920-970)
static void restoreLastStep(OracleModel& m) {
  m.urd = m.urdp;
  m.urdd = m.urddp;
  for (Joint& J : m.joints) J.jVar = J.jVarPrev;
  for (Triad& t : m.triads)
    if (t.nDOFs > 0) std::memcpy(t.ur, t.urPrev, sizeof(M34));
  for (Elem& e : m.elems) {
    std::memcpy(e.supTr, e.supTrPrev, sizeof(M34));
    e.finit = e.finitPrev;
    e.genUr = e.genUrPrev;
  }
}

// One quasi-static load step (staticEquilibriumModule.f90:470-892, staticInt, iop = 0).
static int staticInt(OracleModel& m) {
  const bool pureLinear = m.fixedIt == -1;
  m.time += m.timeStep;
  if (m.fixedIt < 0) {
    restoreLastStep(m);
    m.nIterThisStep = 0;
  }
  updateLoads(m);
  updatePrescribedMotions(m, m.fixedIt < 0);
  // staticIncAndUpdate without increment (linInc = 1): no corotation update
  std::fill(m.rinc.begin(), m.rinc.end(), 0.0);
  if (updateElems(m, false, true, false) != 0) return -1;
  m.nIterThisStep = 0;
  int nSeqNoUpdates = 0;
  for (;;) {
    getForceVectors(m);
    for (int k = 0; k < m.neq; ++k)
      m.residual[k] = (m.fixedIt >= 0 || m.nIterThisStep > 0) ? m.Qk[k] - m.FSk[k] : m.Qk[k];
    m.del = m.residual;
    bool doTangent = m.nIterThisStep < std::max(1, m.nUpdat) || nSeqNoUpdates >= m.maxSeqNoUpdate;
    if (doTangent) {
      bool rhsMotion = m.nIterThisStep == 0 && !m.motions.empty();
      assembleSkyline(m, 0.0, 0.0, 1.0, rhsMotion ? &m.del : nullptr);
      int ierr = skylineFactor(m, 1.0e-12);
      if (ierr < 0) return ierr;
      nSeqNoUpdates = 0;
    } else {
      ++nSeqNoUpdates;
    }
    skylineSolve(m, m.del);
    // staticIncAndUpdate with the increment (linInc = 1 when purely linear)
    expandEq(m, m.del, m.sinc[0], m.nIterThisStep == 0 ? 1.0 : 0.0);
    for (int d = 0; d < m.ndof; ++d) m.rinc[d] += m.sinc[0][d];
    incAll(m, m.sinc[0]);
    if (updateElems(m, false, true, !pureLinear) != 0) return -1;
    std::fill(m.sinc[1].begin(), m.sinc[1].end(), 0.0);
    std::fill(m.sinc[2].begin(), m.sinc[2].end(), 0.0);
    calculateNorms(m);
    m.nIterThisStep++;
    m.nIter++;
    if (pureLinear || m.fixedIt > 0) {
      if (m.nIterThisStep == std::abs(m.fixedIt)) break;
    } else if (m.nIterThisStep > m.maxIt) {
      return 1;
    } else if (m.nIterThisStep >= std::max(2, m.minIt)) {
      if (hasConverged(m)) break;
    }
  }
  getForceVectors(m);
  return 0;
}

// ---------------------------------------------------------------------------
// Set-up (initiateModule.f90:43-547 subset; samSolverModule.f90:95-250)
// ---------------------------------------------------------------------------

// Reads nval doubles from a FEDEM binary matrix file (readDoubleDBfile,
// binaryDBInterface.f90:387-435; writeTagDB/readTagDB, binaryDB.c:643-731):
// the file opens with the tag text '#FEDEM <dtype>', its header ends with the
// version field ';1.0;\n', and the values follow as raw little-endian doubles
// to the end of the file.  The bytes between the tag text and the version
// field (the endian mark and checksum that FFa_writeTag of the fedem-foundation
// submodule writes) are not interpreted.  A relative path is taken relative to
// the directory of the -fsifile option, else the working directory.
static int readFmx(const OracleModel& m, const std::string& name, const char* dtype, size_t nval,
                   std::vector<double>& out) {
  if (name.empty()) return -1;
  std::string path = name;
  const std::string fsiFile = m.opt.s("fsifile");
  if (path[0] != '/' && !fsiFile.empty()) {
    const size_t slash = fsiFile.find_last_of('/');
    if (slash != std::string::npos) path = fsiFile.substr(0, slash + 1) + path;
  }
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return -1;
  std::vector<char> buf;
  char chunk[65536];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  std::fclose(f);
  const std::string tag = std::string("#FEDEM ") + dtype;
  const size_t dataBytes = 8 * nval;
  if (buf.size() < tag.size() + 6 + dataBytes) return -2;
  const size_t head = buf.size() - dataBytes;
  if (std::memcmp(buf.data(), tag.data(), tag.size()) != 0) return -3;
  const std::string ver = ";1.0;\n";
  if (std::memcmp(buf.data() + head - ver.size(), ver.data(), ver.size()) != 0) return -4;
  out.assign(nval, 0.0);
  std::memcpy(out.data(), buf.data() + head, dataBytes);
  return 0;
}

static int setup(OracleModel& m, const char* fsi) {
  std::vector<Record> recs = parseNamelists(fsi);
  for (const Record& r : recs)
    for (const char* bad : {"higher_pair", "mass", "user_el", "tire", "road", "supel_load",
                            "spring_yield", "spring_failure", "master_curve", "friction_set", "bushing_element",
                            "contact_element", "damper_base", "external_control_system", "control_variable",
                            "control_line", "control_input", "control_element", "wind_point", "turbine_config",
                            "master_pos", "generic_part"})
      if (r.name == bad) return -50;  // not in this restatement
  for (const Record& r : recs) {
    if (r.name == "mechanism") {
      m.wDisp[0] = r.d("weighttranslation", 1.0);
      m.wDisp[1] = r.d("weightrotation", 1.0);
      m.wDisp[2] = r.d("weightgeneralized", 1.0);
    } else if (r.name == "environment") {
      auto g = r.dv("gravity");
      for (size_t k = 0; k < 3 && k < g.size(); ++k) m.gravity[k] = g[k];
    } else if (r.name == "triad") {
      Triad t;
      t.id = r.i("id");
      t.nDOFs = r.i("ndofs", 6);
      rowMajor34(r.dv("ur"), t.ur);
      auto bc = r.dv("bc");
      for (size_t k = 0; k < 6 && k < bc.size(); ++k) t.BC[k] = (int)std::lround(bc[k]);
      m.triads.push_back(t);
    } else if (r.name == "element_property") {
      Prop p;
      p.id = r.i("id");
      auto g = r.dv("geometry");
      for (size_t k = 0; k < 8 && k < g.size(); ++k) p.geo[k] = g[k];
      auto mt = r.dv("material");
      for (size_t k = 0; k < 4 && k < mt.size(); ++k) p.mat[k] = mt[k];
      auto o = r.dv("orientation");
      for (size_t k = 0; k < 3 && k < o.size(); ++k) p.orient[k] = o[k];
      m.props.push_back(p);
    } else if (r.name == "function") {
      Func f;
      f.id = r.i("id");
      f.type = r.s("type");
      f.real = r.dv("realdata");
      m.funcs.push_back(f);
    } else if (r.name == "sensor") {
      Sensor sn;
      sn.id = r.i("id");
      sn.type = r.s("type");
      m.sensors.push_back(sn);
    }
  }
  // engines: functionId / argSensorId resolved to indices (engineRoutinesModule.f90)
  for (const Record& r : recs) {
    if (r.name != "engine") continue;
    EngineF en;
    en.id = r.i("id");
    int fid = r.i("functionid", 0), sid = r.i("argsensorid", 0);
    for (size_t k = 0; k < m.funcs.size(); ++k)
      if (m.funcs[k].id == fid) en.func = (int)k;
    for (size_t k = 0; k < m.sensors.size(); ++k)
      if (m.sensors[k].id == sid) en.sensor = (int)k;
    if (fid > 0 && en.func < 0) return -18;
    if (en.func >= 0) {
      std::string t = lower(m.funcs[en.func].type);
      if (t != "scale" && t != "constant" && t != "sinusoidal") return -19;  // other function types are not in this subset
    }
    m.engines.push_back(en);
  }
  auto findEngine = [&m](int id) {
    for (size_t k = 0; k < m.engines.size(); ++k)
      if (m.engines[k].id == id) return (int)k;
    return -1;
  };
  // superelements and their undeformed triad positions
  int pendingUnd = -1;
  std::vector<Axial> springs, dampers;
  for (const Record& r : recs) {
    if (r.name == "sup_el") {
      // SUP_EL namelist (supElTypeModule.f90:1299-1350) as ReadSupEls uses it
      // (initiateSupElTypeModule.f90:140-700)
      Elem e;
      e.id = r.i("id");
      auto tids = r.dv("triadids");
      e.nTri = r.i("numtriads", 2);
      e.nGen = r.i("numgendofs", 0);
      if (e.nTri < 2 || (int)tids.size() < e.nTri || e.nGen < 0) return -10;
      // not in this restatement: nonlinear parts, part load cases, stress
      // stiffening, mass-matrix correction, the shadowPosAlg 2 frame,
      // time-dependent stiffness or damping scaling
      if (r.i("numstates", 0) > 0 || r.i("numloadcase", 0) > 0) return -10;
      for (double v : r.dv("stressstiffflag"))
        if (v > 0.0) return -10;
      if (r.i("masscorrflag", -1) > 0 || r.i("shadowposalg", 0) > 1) return -10;
      if (r.i("stiffengineid", 0) > 0 || r.i("strdmpengineid", 0) > 0) return -10;
      e.tri.assign(e.nTri, -1);
      for (int k = 0; k < e.nTri; ++k) {
        e.tri[k] = findTriad(m, (int)std::lround(tids[k]));
        if (e.tri[k] < 0) return -11;
      }
      int refIds[3] = {r.i("reftriad1id"), r.i("reftriad2id"), r.i("reftriad3id")};
      for (int j = 0; j < 3; ++j) {
        e.ref[j] = -1;
        for (int k = 0; k < e.nTri; ++k)
          if ((int)std::lround(tids[k]) == refIds[j]) e.ref[j] = k;
        if (e.ref[j] < 0) return -12;
      }
      e.TrUnd.assign(12 * (size_t)e.nTri, 0.0);
      if (const auto* f = r.get("inputfiles"))
        for (size_t k = 0; k < 3 && k < f->size(); ++k) e.files[k] = (*f)[k];
      auto bcg = r.dv("bc"), a3 = r.dv("alpha3"), a4 = r.dv("alpha4");
      for (int g = 0; g < e.nGen; ++g) {
        e.genBC.push_back(g < (int)bcg.size() ? (int)std::lround(bcg[g]) : 1);
        e.alpha3.push_back(g < (int)a3.size() ? a3[g] : 0.0);
        e.alpha4.push_back(g < (int)a4.size() ? a4[g] : 0.0);
      }
      std::vector<double> off[3] = {r.dv("offset1"), r.dv("offset2"), r.dv("offset3")};
      rowMajor34(r.dv("suppos"), e.supTr);
      e.stiffScale = r.d("stiffscale", 1.0);
      e.massScale = r.d("massscale", 1.0);
      e.alpha1 = r.d("alpha1", 0.0);
      e.alpha2 = r.d("alpha2", 0.0);
      // TransformOffset (supElTypeModule.f90:779-789)
      for (int j = 0; j < 3; ++j) {
        double o[3] = {0, 0, 0};
        for (size_t k = 0; k < 3 && k < off[j].size(); ++k) o[k] = off[j][k];
        double so[3];
        for (int q = 0; q < 3; ++q) so[q] = e.supTr[q][0] * o[0] + e.supTr[q][1] * o[1] + e.supTr[q][2] * o[2];
        const Triad& t = m.triads[e.tri[e.ref[j]]];
        for (int c = 0; c < 3; ++c) e.offset[j][c] = so[0] * t.ur[0][c] + so[1] * t.ur[1][c] + so[2] * t.ur[2][c];
      }
      if (e.files[0].empty()) {  // a beam: matrices from its element property
        int pid = r.i("elpropid");
        for (size_t k = 0; k < m.props.size(); ++k)
          if (m.props[k].id == pid) e.prop = (int)k;
        if (e.prop < 0 || e.nTri != 2 || e.nGen != 0) return -13;
      }
      m.elems.push_back(e);
      pendingUnd = (int)m.elems.size() - 1;
    } else if (r.name == "triad_undpos") {
      int sid = r.i("supelid"), tid = r.i("triadid");
      int ei = -1;
      for (int k = (int)m.elems.size() - 1; k >= 0; --k)
        if (m.elems[k].id == sid) { ei = k; break; }
      if (ei < 0) return -14;
      Elem& e = m.elems[ei];
      int node = -1;
      for (int k = 0; k < e.nTri; ++k)
        if (m.triads[e.tri[k]].id == tid) node = k;
      if (node < 0) return -15;
      for (const char* key : {"eccvec", "eccmass"})
        for (double v : r.dv(key))
          if (std::fabs(v) > 1.0e-16) return -15;  // eccentricity vectors are not in this restatement
      M34 U;
      rowMajor34(r.dv("undposinsupelsystem"), U);
      for (int rr = 0; rr < 3; ++rr)
        for (int c = 0; c < 4; ++c) e.TrUnd[12 * node + 4 * rr + c] = U[rr][c];
    } else if (r.name == "load") {
      Load l;
      l.triad = findTriad(m, r.i("triadid"));
      if (l.triad < 0) return -16;
      l.dof = r.i("ldof");
      if (l.dof < 1 || l.dof > 6) return -17;
      l.f0 = r.d("f0");
      l.f1 = r.d("f1");
      int eid = r.i("loadengineid", 0);
      if (eid > 0 && (l.engine = findEngine(eid)) < 0) return -18;
      m.loads.push_back(l);
    } else if (r.name == "spring_element") {
      auto tids = r.dv("triadids");
      auto sb = r.dv("springbaseid");
      int nb = 0;
      for (double v : sb) nb += v > 0.0;
      if (tids.size() < 2 || tids[1] <= 0.0 || (tids.size() > 2 && tids[2] > 0.0) || nb != 1 || sb[0] <= 0.0)
        return -40;  // axial springs between two triads only
      Axial a;
      a.kind = 0;
      for (int k = 0; k < 2; ++k)
        if ((a.tri[k] = findTriad(m, (int)std::lround(tids[k]))) < 0) return -41;
      a.alpha2 = r.d("alpha2");
      int bid = (int)std::lround(sb[0]);
      bool found = false;
      for (const Record& q : recs) {
        if (q.name != "spring_base" || q.i("id") != bid) continue;
        if (q.i("stifffuncid") > 0 || q.i("forcefuncid") > 0 || q.i("lengthengineid") > 0 ||
            q.i("stiffscaleengineposid") > 0 || q.i("stiffscaleenginenegid") > 0 || q.i("springfailureid") > 0 ||
            q.i("springyieldid") > 0)
          return -42;  // constant linear springs only
        a.s0 = q.d("s0");
        a.l0 = q.d("l0");
        found = true;
      }
      if (!found) return -43;
      springs.push_back(a);
    } else if (r.name == "damper") {
      Axial a;
      a.kind = 1;
      int t1 = r.i("triad1id"), t2 = r.i("triad2id");
      if (t1 <= 0 || t2 <= 0) return -44;  // axial dampers only
      if (r.i("coeffscaleengineid") > 0 || r.i("coefffuncid") > 0 || r.i("forcefuncid") > 0) return -45;
      if ((a.tri[0] = findTriad(m, t1)) < 0 || (a.tri[1] = findTriad(m, t2)) < 0) return -46;
      // the triad with most DOFs is triad 1 (initiateDamperTypeModule.f90:160-165)
      if (m.triads[a.tri[0]].nDOFs < m.triads[a.tri[1]].nDOFs) std::swap(a.tri[0], a.tri[1]);
      a.d0 = r.d("d0");
      dampers.push_back(a);
    } else if (r.name == "motion") {
      Motion mo;
      mo.triad = findTriad(m, r.i("triadid"));
      if (mo.triad < 0) return -16;
      mo.dof = r.i("ldof");
      if (mo.dof < 1 || mo.dof > 6) return -17;
      std::string t = lower(r.s("type"));
      if (!t.empty() && t != "deflection") return -19;  // velocity/acceleration motions are not in this subset
      mo.d0 = r.d("d0");
      mo.d1 = r.d("d1");
      int eid = r.i("motionengineid", 0);
      if (eid > 0 && (mo.engine = findEngine(eid)) < 0) return -18;
      m.motions.push_back(mo);
    }
  }
  (void)pendingUnd;
  // master-slave joints (initiateJointTypeModule.f90:120-600): one master
  // triad, joint variables JointVarDefs = (lDof, iMat) pairs with at most one
  // rotation per position matrix, no joint springs, dampers or friction
  for (const Record& r : recs) {
    if (r.name != "masterslavejoint") continue;
    Joint J;
    J.id = r.i("id");
    J.type = r.i("type");
    if (J.type != 1 && J.type != 3 && J.type != 4) return -70;  // revolute, rigid, free (point-to-point)
    if (r.i("version") < 0) return -70;
    J.slave = findTriad(m, r.i("slaveid"));
    J.master = findTriad(m, r.i("masterid"));
    if (J.slave < 0 || J.master < 0 || J.slave == J.master) return -71;
    if (m.triads[J.slave].nDOFs != 6) return -72;
    const int nv = r.i("njointvars", 0);
    auto defs = r.dv("jointvardefs"), bc = r.dv("bc"), v0 = r.dv("jvarinitval");
    for (const char* key : {"springid", "damperid", "frictionsetid", "frictionspringid", "frictionengineid"})
      for (double v : r.dv(key))
        if (v > 0.0) return -73;
    for (int k = 0; k < nv; ++k) {
      const int ld = 2 * k < (int)defs.size() ? (int)std::lround(defs[2 * k]) : 0;
      const int im = 2 * k + 1 < (int)defs.size() ? (int)std::lround(defs[2 * k + 1]) : 0;
      if (ld < 1 || ld > 6 || im < 1) return -74;
      J.lDof.push_back(ld);
      J.iMat.push_back(im);
      J.BC.push_back(k < (int)bc.size() ? (int)std::lround(bc[k]) : 1);
      J.jVar.push_back(k < (int)v0.size() ? v0[k] : 0.0);
      J.nMats = std::max(J.nMats, im);
    }
    for (int im = 1; im <= J.nMats; ++im) {
      int nrot = 0;
      for (int k = 0; k < nv; ++k) nrot += J.iMat[k] == im && J.lDof[k] > 3;
      if (nrot > 1) return -75;  // several rotations in one level need dOmega/dTheta
    }
    J.jVarPrev = J.jVar;
    // joint position: initPosInGlobal row by row, rotation re-orthonormalised
    auto pg = r.dv("initposinglobal");
    rowMajor34(pg, J.JPosInG);
    {
      double R[3][3];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) R[a][b] = J.JPosInG[a][b];
      orthonorm3(R);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) J.JPosInG[a][b] = R[a][b];
    }
    M34 inv, tmp;
    invert34(J.JPosInG, inv);
    matmul34(inv, m.triads[J.slave].ur, J.STPos0InJ);
    for (int im = J.nMats; im >= 1; --im) {
      M34 F, Fi;
      jointPosFromVars(J, im, F);
      invert34(F, Fi);
      matmul34(Fi, J.STPos0InJ, tmp);
      std::memcpy(J.STPos0InJ, tmp, sizeof(M34));
    }
    invert34(m.triads[J.master].ur, inv);
    matmul34(inv, J.JPosInG, J.JPosInT);
    J.nM = std::min(6, m.triads[J.master].nDOFs);
    J.ncol = J.nM + nv;
    J.T.assign(6 * (size_t)J.ncol, 0.0);
    m.joints.push_back(J);
  }
  for (size_t a = 0; a < m.joints.size(); ++a)
    for (size_t b = 0; b < m.joints.size(); ++b)
      if (a != b && (m.joints[a].slave == m.joints[b].slave || m.joints[a].master == m.joints[b].slave))
        return -76;  // a triad dependent twice, or chained joints
  if (!m.joints.empty() && !m.motions.empty()) return -77;  // joints with prescribed motions: not in this subset
  m.axials = springs;
  m.axials.insert(m.axials.end(), dampers.begin(), dampers.end());
  for (const Axial& a : m.axials)
    for (int k = 0; k < 2; ++k)
      if (m.triads[a.tri[k]].nDOFs < 3) return -47;
  // element matrices: reduced parts from their matrix files (ReadSupElMatrices,
  // initiateSupElTypeModule.f90:962-1033), beams from their cross section
  // (finiteElementModule.f90:283-541, CalcBeamElementMatrices)
  for (Elem& e : m.elems) {
    e.allocate();
    if (e.prop < 0) {
      const size_t nn = (size_t)e.n * e.n;
      if (readFmx(m, e.files[0], "stiffness matrix", nn, e.K) != 0) return -80;
      if (readFmx(m, e.files[1], "mass matrix", nn, e.M) != 0) return -81;
      if (!e.files[2].empty() && readFmx(m, e.files[2], "gravity force vectors", 3 * (size_t)e.n, e.fg) != 0)
        return -82;
      // structural damping (computeStructDamping, :740-780): Rayleigh on the
      // unscaled matrices, individual factors on the generalized DOFs
      bool haveM = e.alpha1 > 0.0, haveK = e.alpha2 > 0.0;
      for (int g = 0; g < e.nGen; ++g) {
        haveM = haveM || e.alpha3[g] > 0.0;
        haveK = haveK || e.alpha4[g] > 0.0;
      }
      bool any3 = false, any4 = false;
      for (int g = 0; g < e.nGen; ++g) {
        any3 = any3 || e.alpha3[g] > 0.0;
        any4 = any4 || e.alpha4[g] > 0.0;
      }
      for (int g = 0; g < e.nGen; ++g) {
        if (!any3) e.alpha3[g] = e.alpha1;
        if (!any4) e.alpha4[g] = e.alpha2;
      }
      const int n = e.n, nd = 6 * e.nTri;
      if (haveM || haveK) {
        for (size_t k = 0; k < nn; ++k) e.C[k] = e.alpha1 * e.M[k] + e.alpha2 * e.K[k];
        for (int g = 0; g < e.nGen; ++g) {
          const int j = nd + g;
          const double d3 = e.alpha3[g] - e.alpha1, d4 = e.alpha4[g] - e.alpha2;
          if (std::fabs(d3) > 1.0e-16) {
            e.C[j + (size_t)n * j] += d3 * e.M[j + (size_t)n * j];
            for (int i = 0; i < nd; ++i) e.C[i + (size_t)n * j] += d3 * e.M[i + (size_t)n * j];
            for (int i = 0; i < nd; ++i) e.C[j + (size_t)n * i] += d3 * e.M[j + (size_t)n * i];
          }
          if (std::fabs(d4) > 1.0e-16) e.C[j + (size_t)n * j] += d4 * e.K[j + (size_t)n * j];
        }
        e.hasC = true;
      }
      if (std::fabs(e.stiffScale - 1.0) > 1.0e-16)
        for (size_t k = 0; k < nn; ++k) e.K[k] *= e.stiffScale;
      if (std::fabs(e.massScale - 1.0) > 1.0e-16) {
        for (size_t k = 0; k < nn; ++k) e.M[k] *= e.massScale;
        for (int k = 0; k < 3 * n; ++k) e.fg[k] *= e.massScale;
      }
      double a2 = e.alpha2;
      if (e.hasC && std::fabs(e.stiffScale - 1.0) > 1.0e-16) a2 /= e.stiffScale;
      e.kDmp = a2;
      e.hasVld = a2 > 0.0 && m.stiffDampFiltering > 0;
      if (updateCorot(m, e, true) != 0) return -22;
      std::memcpy(e.supTrPrev, e.supTr, sizeof(M34));
      continue;
    }
    const Prop& p = m.props[e.prop];
    e.kDmp = 0.0;
    double Xg[5][3];
    for (int k = 0; k < 3; ++k) {
      Xg[3][k] = e.tu(0, k, 3);
      Xg[4][k] = e.tu(1, k, 3);
      Xg[0][k] = Xg[3][k];
      Xg[1][k] = Xg[4][k];
    }
    bool hasZ = std::fabs(p.orient[0]) > epsDiv0 || std::fabs(p.orient[1]) > epsDiv0 || std::fabs(p.orient[2]) > epsDiv0;
    if (!hasZ) {
      double v[3] = {Xg[1][0] - Xg[0][0], Xg[1][1] - Xg[0][1], Xg[1][2] - Xg[0][2]}, T[3][3];
      if (trans1V(v, T) != 0) return -20;
      for (int k = 0; k < 3; ++k) Xg[2][k] = Xg[0][k] + T[k][2];
    } else {
      for (int k = 0; k < 3; ++k) Xg[2][k] = Xg[0][k] + p.orient[k];
    }
    double X[5], Y[5], Z[5];
    for (int q = 0; q < 5; ++q) { X[q] = Xg[q][0]; Y[q] = Xg[q][1]; Z[q] = Xg[q][2]; }
    double EP[6] = {p.mat[1], p.mat[2], p.geo[0], p.geo[1], p.geo[2], p.geo[3]};
    double CA[2] = {p.geo[4], p.geo[5]}, XS[2] = {p.geo[6], p.geo[7]};
    if (beam31(e.K.data(), X, Y, Z, EP, CA, XS) != 0) return -21;
    double rho = p.mat[0];
    double Ix = p.geo[1] + p.geo[2];
    if (Ix <= 0.0) Ix = p.geo[3];
    double Area = EP[2], z1 = Ix;
    if (EP[0] <= epsDiv0 && rho > epsDiv0) { Area = 1.0; z1 = Ix / rho; }
    beam35(e.M.data(), X, Y, Z, Area, rho, z1);
    for (int i = 0; i < 12; ++i)
      for (int c = 0; c < 3; ++c) e.fg[i + 12 * c] = e.M[i + 12 * c] + e.M[i + 12 * (c + 6)];
    // structural damping (initiateSupElTypeModule.f90:549-599), unscaled matrices
    bool damp = e.alpha1 > 0.0 || e.alpha2 > 0.0;
    if (damp) {
      for (int k = 0; k < 144; ++k) e.C[k] = e.alpha1 * e.M[k] + e.alpha2 * e.K[k];
      e.hasC = true;
    }
    if (std::fabs(e.stiffScale - 1.0) > 1.0e-16)
      for (int k = 0; k < 144; ++k) e.K[k] *= e.stiffScale;
    if (std::fabs(e.massScale - 1.0) > 1.0e-16) {
      for (int k = 0; k < 144; ++k) e.M[k] *= e.massScale;
      for (int k = 0; k < 36; ++k) e.fg[k] *= e.massScale;
    }
    double a1 = e.alpha1, a2 = e.alpha2;
    if (damp && std::fabs(e.massScale - 1.0) > 1.0e-16) a1 /= e.massScale;
    if (damp && std::fabs(e.stiffScale - 1.0) > 1.0e-16) a2 /= e.stiffScale;
    e.kDmp = a2;
    e.hasVld = a2 > 0.0 && m.stiffDampFiltering > 0;
    (void)a1;
    if (updateCorot(m, e, true) != 0) return -22;
    std::memcpy(e.supTrPrev, e.supTr, sizeof(M34));
  }
  // SAM (samSolverModule.f90:95-250): triads in input order, MSC = BC,
  // equations numbered over the free DOFs in DOF order
  m.ndof = 0;
  for (Triad& t : m.triads) {
    t.firstDof = m.ndof;
    m.ndof += t.nDOFs;
    std::memcpy(t.urPrev, t.ur, sizeof(M34));
  }
  const int ntriDof = m.ndof;
  for (Elem& e : m.elems) {  // generalized DOFs of the parts after the triads (initSAM_dofStatus)
    if (e.nGen == 0) continue;
    e.genFirstDof = m.ndof;
    m.ndof += e.nGen;
  }
  for (Joint& J : m.joints) {  // joint DOFs after those
    J.firstDof = m.ndof;
    m.ndof += (int)J.lDof.size();
  }
  m.meqn.assign(m.ndof, 0);
  m.dofType.assign(m.ndof, 1);
  m.dep.assign(m.ndof, -1);
  m.neq = 0;
  for (size_t j = 0; j < m.joints.size(); ++j) {
    const Triad& st = m.triads[m.joints[j].slave];
    for (int k = 0; k < 6; ++k) {
      if (st.BC[k] != 1) return -78;  // a dependent DOF must be free
      m.dep[st.firstDof + k] = 6 * (int)j + k;
    }
  }
  // BC 2 (fixed during initial equilibrium only) counts as free unless the
  // initial equilibrium iterations are on (initiateTriadTypeModule.f90:57-123)
  const bool addBC = m.opt.b("initEquilibrium", false);
  std::vector<int> prescribed(m.ndof, 0);
  for (size_t k = 0; k < m.motions.size(); ++k) {
    Motion& mo = m.motions[k];
    int d = m.triads[mo.triad].firstDof + mo.dof - 1;
    if (mo.dof > m.triads[mo.triad].nDOFs || prescribed[d]) return -32;
    mo.iceq = (int)k + 1;
    prescribed[d] = mo.iceq;
  }
  for (Triad& t : m.triads)
    for (int k = 0; k < t.nDOFs; ++k) {
      int d = t.firstDof + k;
      m.dofType[d] = k < 3 ? 1 : 2;
      if (m.dep[d] >= 0) continue;  // dependent (joint slave) DOF: no equation
      if (prescribed[d]) m.meqn[d] = -prescribed[d];  // MEQN = -ICEQ (samSolverModule.f90)
      else if (t.BC[k] == 1 || (t.BC[k] == 2 && !addBC)) m.meqn[d] = ++m.neq;
      else if (t.BC[k] != 0) return -30;  // additional initial-equilibrium BCs are not in this subset
    }
  for (Elem& e : m.elems)
    for (int g = 0; g < e.nGen; ++g) {
      const int d = e.genFirstDof + g;
      m.dofType[d] = 3;  // genDof_p
      if (e.genBC[g] == 1 || (e.genBC[g] == 2 && !addBC)) m.meqn[d] = ++m.neq;
      else if (e.genBC[g] != 0) return -30;
    }
  for (Joint& J : m.joints)
    for (size_t k = 0; k < J.lDof.size(); ++k) {
      const int d = J.firstDof + (int)k;
      m.dofType[d] = J.lDof[k] <= 3 ? 1 : 2;
      if (J.BC[k] == 1 || (J.BC[k] == 2 && !addBC)) m.meqn[d] = ++m.neq;
      else if (J.BC[k] != 0) return -30;
    }
  (void)ntriDof;
  for (Joint& J : m.joints) {
    J.colEq.assign(J.ncol, -1);
    for (int c = 0; c < J.nM; ++c) J.colEq[c] = m.meqn[m.triads[J.master].firstDof + c] - 1;
    for (size_t k = 0; k < J.lDof.size(); ++k) J.colEq[J.nM + k] = m.meqn[J.firstDof + k] - 1;
    for (int c = 0; c < J.ncol; ++c)
      if (J.colEq[c] < -1) return -77;  // prescribed master DOF
  }
  for (const Axial& a : m.axials)
    for (int k = 0; k < 2; ++k)
      if (m.dep[m.triads[a.tri[k]].firstDof] >= 0) return -79;  // axial element on a dependent triad
  for (const Load& l : m.loads)
    if (m.dep[m.triads[l.triad].firstDof] >= 0) return -79;  // load on a dependent triad
  m.ccv.assign(m.motions.size(), 0.0);
  for (const Elem& e : m.elems)
    for (int k = 0; k < e.nTri; ++k)
      if (m.triads[e.tri[k]].nDOFs != 6) return -31;
  m.elOff.assign(m.elems.size() + 1, 0);
  for (size_t k = 0; k < m.elems.size(); ++k) m.elOff[k + 1] = m.elOff[k] + m.elems[k].n;
  m.elEq.assign(m.elOff.back(), -1);
  for (size_t k = 0; k < m.elems.size(); ++k)
    for (int i = 0; i < m.elems[k].n; ++i) m.elEq[m.elOff[k] + i] = m.meqn[elemDof(m, m.elems[k], i)] - 1;
  m.axEq.assign(6 * m.axials.size(), -1);
  for (size_t k = 0; k < m.axials.size(); ++k)
    for (int n = 0; n < 2; ++n)
      for (int d = 0; d < 3; ++d) m.axEq[6 * k + 3 * n + d] = m.meqn[m.triads[m.axials[k].tri[n]].firstDof + d] - 1;
  // skyline profile and CSR upper pattern
  m.first.resize(m.neq);
  for (int j = 0; j < m.neq; ++j) m.first[j] = j;
  std::vector<std::vector<int>> rows(m.neq);
  auto clique = [&](const int* eq, int n) {
    for (int i = 0; i < n; ++i) {
      if (eq[i] < 0) continue;
      for (int j = 0; j < n; ++j) {
        if (eq[j] < eq[i]) continue;
        m.first[eq[j]] = std::min(m.first[eq[j]], eq[i]);
        rows[eq[i]].push_back(eq[j]);
      }
    }
  };
  for (size_t k = 0; k < m.elems.size(); ++k) {
    if (!elemConstrained(m, m.elems[k])) {
      clique(&m.elEq[m.elOff[k]], m.elems[k].n);
      continue;
    }
    // every equation the element's DOFs expand to (the coefficients vary)
    std::vector<int> ex;
    for (int n = 0; n < m.elems[k].nTri; ++n) {
      const Triad& t = m.triads[m.elems[k].tri[n]];
      const int d0 = t.firstDof;
      if (m.dep[d0] >= 0) {
        const Joint& J = m.joints[m.dep[d0] / 6];
        for (int c = 0; c < J.ncol; ++c) ex.push_back(J.colEq[c]);
      } else {
        for (int q = 0; q < 6; ++q) ex.push_back(m.meqn[d0 + q] - 1);
      }
    }
    for (int g = 0; g < m.elems[k].nGen; ++g) ex.push_back(m.meqn[m.elems[k].genFirstDof + g] - 1);
    clique(ex.data(), (int)ex.size());
  }
  for (size_t k = 0; k < m.axials.size(); ++k) clique(&m.axEq[6 * k], 6);
  m.colptr.resize(m.neq + 1);
  m.colptr[0] = 0;
  for (int j = 0; j < m.neq; ++j) m.colptr[j + 1] = m.colptr[j] + (j - m.first[j] + 1);
  m.sky.assign(m.colptr[m.neq], 0.0);
  m.rowptr.assign(m.neq + 1, 0);
  m.cols.clear();
  for (int i = 0; i < m.neq; ++i) {
    auto& r = rows[i];
    r.push_back(i);
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    m.rowptr[i + 1] = m.rowptr[i] + (int)r.size();
    m.cols.insert(m.cols.end(), r.begin(), r.end());
  }
  // system vectors
  m.urd.assign(m.ndof, 0.0);
  m.urdd.assign(m.ndof, 0.0);
  m.urdp.assign(m.ndof, 0.0);
  m.urddp.assign(m.ndof, 0.0);
  m.dk.assign(m.ndof, 0.0);
  m.ak.assign(m.ndof, 0.0);
  m.rinc.assign(m.ndof, 0.0);
  for (auto& s : m.sinc) s.assign(m.ndof, 0.0);
  m.FSk.assign(m.neq, 0.0);
  m.FDk.assign(m.neq, 0.0);
  m.FIk.assign(m.neq, 0.0);
  m.Qk.assign(m.neq, 0.0);
  m.FIactual.assign(m.neq, 0.0);
  m.residual.assign(m.neq, 0.0);
  m.del.assign(m.neq, 0.0);
  return 0;
}

static void readControl(OracleModel& m) {
  const Options& o = m.opt;
  // initiateSystemTypeModule.f90:41-185
  double a = o.d("alphaNewmark", 0.1);
  if (a < 0.0) a = 0.0;
  if (a > 1.0 / 3.0) a = 1.0 / 3.0;
  m.alpha = -a;
  m.beta = (1.0 - m.alpha) * (1.0 - m.alpha) / 4.0;
  m.gamma = 0.5 - m.alpha;
  m.tStart = o.d("timeStart", 0.0);
  m.tEnd = o.d("timeEnd", 0.0);
  m.tInc = o.d("timeInc", 0.0);
  m.minInc = o.d("minInc", 0.001);
  if (m.tInc < 1.0e-6) m.tInc = 1.0e-6;
  m.maxIt = o.i("maxit", 15);
  m.minIt = o.i("minit", 1);
  m.fixedIt = o.i("numit", 0);
  m.nUpdat = o.i("nupdat", 0);
  m.maxSeqNoUpdate = o.i("maxSeqNoUpdate", 100);
  m.tolUpdateFactor = o.d("tolUpdateFactor", 0.0);
  m.stiffDampFiltering = o.i("stiffDampFiltering", 1);
  m.tQStatic = o.d("quasiStatic", 0.0);
  if (m.tQStatic <= m.tStart) m.tQStatic = -1.0e99;  // no quasi-static increments
  for (int k = 0; k < 3; ++k) m.wForce[k] = m.wDisp[k] > 0.0 ? 1.0 / m.wDisp[k] : 0.0;
  initTol(o, "tolDispNorm", m.dis[0]);
  initTol(o, "tolDispTra", m.dis[1]);
  initTol(o, "tolDispRot", m.dis[2]);
  initTol(o, "tolDispGen", m.dis[3]);
  initTol(o, "tolVelNorm", m.vel[0]);
  initTol(o, "tolVelTra", m.vel[1]);
  initTol(o, "tolVelRot", m.vel[2]);
  initTol(o, "tolVelGen", m.vel[3]);
  initTol(o, "tolAccNorm", m.acc[0]);
  initTol(o, "tolAccTra", m.acc[1]);
  initTol(o, "tolAccRot", m.acc[2]);
  initTol(o, "tolAccGen", m.acc[3]);
  initTol(o, "tolResNorm", m.res[0]);
  initTol(o, "tolResTra", m.res[1]);
  initTol(o, "tolResRot", m.res[2]);
  initTol(o, "tolResGen", m.res[3]);
  initTol(o, "tolEnerMax", m.ener[0]);
  initTol(o, "tolEnerSum", m.ener[1]);
}

static bool hasReached(const OracleModel& m, double t) { return m.time + 0.1 * m.minInc > t; }

// systemTypeModule.f90:334-347
static bool isQuasiStatic(const OracleModel& m, double t) { return t < m.tQStatic + 0.1 * m.minInc; }

}  // namespace

// ===========================================================================
// C interface
// ===========================================================================

extern "C" OracleModel* oracle_create(const char* fsi, int argc, const char* const* argv, int* ierr) {
  OracleModel* m = new OracleModel();
  m->opt.parse(argc, argv);
  int err = 0;
  if (!fsi) err = -1;
  if (!err) err = setup(*m, fsi);
  if (!err) {
    readControl(*m);
    m->time = m->tStart;
    m->timeStep = m->tInc;
    // updateLoads at the start time, static equilibrium, initial force vectors
    updateLoads(*m);
    err = staticEquilibrium(*m);
    if (!err) getForceVectors(*m);
    // motions take their start-time values without moving the triads
    // (updatePrescribedMotionsB, motionRoutinesModule.f90:213-245)
    for (Motion& mo : m->motions) {
      mo.D = mo.engine >= 0 ? mo.d0 + mo.d1 * engineValue(*m, mo.engine) : mo.d0;
      if (!err && m->opt.b("initEquilibrium", false) && mo.D != 0.0) err = -33;  // not in this subset
    }
  }
  if (err) {
    delete m;
    if (ierr) *ierr = err;
    return nullptr;
  }
  for (const Triad& t : m->triads)
    for (int r = 0; r < 3; ++r) m->x0.push_back(t.ur[r][3]);
  if (ierr) *ierr = 0;
  return m;
}

extern "C" void oracle_destroy(OracleModel* m) { delete m; }

extern "C" double oracle_get_max_displacement(OracleModel* m) { return m ? m->maxDisp : 0.0; }

// solverModule.f90:658-1000, solveStep (fixed step size, no quasi-static range)
extern "C" int oracle_solve_next(OracleModel* m, int* ierr) {
  if (ierr) *ierr = 0;
  if (!m || m->error) { if (ierr) *ierr = m ? m->error : -1; return 0; }
  if (m->tStart <= m->tEnd && hasReached(*m, m->tEnd)) return 0;
  m->timeStep = m->tInc;
  // quasi-static load steps up to the quasiStatic time, Newmark after it
  // (solverModule.f90:826-860)
  bool linearStatic = false;
  int err = 0;
  if (isQuasiStatic(*m, m->time + m->timeStep)) {
    m->quasiSteps++;
    err = staticInt(*m);
    linearStatic = m->fixedIt < 0;
  } else {
    if (m->quasiSteps > 0) {
      // continuing with dynamics: estimate the starting velocity
      for (int d = 0; d < m->ndof; ++d) m->urd[d] = m->rinc[d] / m->timeStep;
      m->quasiSteps = 0;
    }
    err = newmarkInt(*m);
  }
  if (err != 0) { m->error = err; if (ierr) *ierr = err; return 0; }
  m->nStep++;
  bool finished = m->tStart <= m->tEnd && hasReached(*m, m->tEnd);
  // terminateStep (solverRoutinesModule.f90:728-827)
  for (Triad& t : m->triads) {
    if (t.nDOFs == 6) {
      double R[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[r][c] = t.ur[r][c];
      orthonorm3(R);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t.ur[r][c] = R[r][c];
    }
  }
  if (!finished && !linearStatic) {
    m->urdp = m->urd;
    m->urddp = m->urdd;
    for (Triad& t : m->triads) std::memcpy(t.urPrev, t.ur, sizeof(M34));
    for (Elem& e : m->elems) {
      std::memcpy(e.supTrPrev, e.supTr, sizeof(M34));
      e.finitPrev = e.finit;
      e.genUrPrev = e.genUr;
    }
    for (Joint& J : m->joints) J.jVarPrev = J.jVar;
  }
  for (size_t k = 0; k < m->triads.size(); ++k)
    for (int r = 0; r < 3; ++r) m->maxDisp = std::max(m->maxDisp, std::fabs(m->triads[k].ur[r][3] - m->x0[3 * k + r]));
  m->finished = finished;
  return finished ? 0 : 1;
}

extern "C" int oracle_get_state_var(OracleModel* m, int id, double* var) {
  if (!m) return 0;
  int k = findTriad(*m, id);
  if (k < 0 || m->triads[k].nDOFs < 3) return 0;
  for (int r = 0; r < 3; ++r) var[r] = m->triads[k].ur[r][3];
  return 3;
}

extern "C" double oracle_get_time(OracleModel* m) { return m ? m->time : 0.0; }
extern "C" int oracle_get_ndof(OracleModel* m) { return m ? m->ndof : 0; }
extern "C" int oracle_get_neq(OracleModel* m) { return m ? m->neq : 0; }
extern "C" int oracle_get_ntriads(OracleModel* m) { return m ? (int)m->triads.size() : 0; }
extern "C" int oracle_get_nelements(OracleModel* m) { return m ? (int)m->elems.size() : 0; }

extern "C" int oracle_get_meqn(OracleModel* m, int* meqn) {
  if (!m) return 0;
  for (int d = 0; d < m->ndof; ++d) meqn[d] = m->meqn[d];
  return m->ndof;
}

extern "C" int oracle_get_triad_ur(OracleModel* m, double* ur) {
  if (!m) return 0;
  for (size_t k = 0; k < m->triads.size(); ++k)
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 3; ++r) ur[12 * k + 3 * c + r] = m->triads[k].ur[r][c];
  return (int)m->triads.size();
}

extern "C" long long oracle_get_iterations(OracleModel* m) { return m ? m->nIter : 0; }

extern "C" int oracle_get_last_norms(OracleModel* m, double* n4) {
  if (!m) return 0;
  for (int k = 0; k < 4; ++k) n4[k] = m->lastNorms[k];
  return m->nIterThisStep;
}

extern "C" int oracle_get_csr_pattern(OracleModel* m, int* rowptr, int* cols) {
  if (!m) return 0;
  if (rowptr) std::copy(m->rowptr.begin(), m->rowptr.end(), rowptr);
  if (cols) std::copy(m->cols.begin(), m->cols.end(), cols);
  return (int)m->cols.size();
}

extern "C" int oracle_assemble_newton(OracleModel* m, double sM, double sC, double sK, double* values) {
  if (!m) return 0;
  std::fill(values, values + m->cols.size(), 0.0);
  std::vector<double> Ns, Nl;
  for (size_t k = 0; k < m->elems.size(); ++k) {
    const Elem& e = m->elems[k];
    const int n = e.n;
    Ns.resize((size_t)n * n);
    Nl.resize((size_t)n * n);
    for (int q = 0; q < n * n; ++q) {
      double v = sM * e.M[q];
      if (e.hasC) v += sC * e.stifScl * e.C[q];
      v += sK * e.stifScl * e.K[q];
      Nl[q] = v;
    }
    rotatedElementMatrix(e, Nl.data(), Ns.data());
    const int* eq = &m->elEq[m->elOff[k]];
    auto add = [&](int a, int b, double v) {
      const int* lo = &m->cols[m->rowptr[a]];
      const int* en = &m->cols[0] + m->rowptr[a + 1];
      values[std::lower_bound(lo, en, b) - &m->cols[0]] += v;
    };
    if (elemConstrained(*m, e)) {
      std::vector<Term> ti, tj;
      for (int i = 0; i < n; ++i) {
        dofTerms(*m, elemDof(*m, e, i), ti);
        for (int j = 0; j < n; ++j) {
          dofTerms(*m, elemDof(*m, e, j), tj);
          for (const Term& a : ti)
            for (const Term& b : tj)
              if (b.eq >= a.eq) add(a.eq, b.eq, a.c * b.c * Ns[i + (size_t)n * j]);
        }
      }
      continue;
    }
    for (int i = 0; i < n; ++i) {
      if (eq[i] < 0) continue;
      for (int j = 0; j < n; ++j) {
        if (eq[j] < eq[i]) continue;
        add(eq[i], eq[j], Ns[i + (size_t)n * j]);
      }
    }
  }
  for (size_t k = 0; k < m->axials.size(); ++k) {
    double A[9];
    axialBlock(m->axials[k], sC, sK, A);
    const int* eq = &m->axEq[6 * k];
    for (int i = 0; i < 6; ++i) {
      if (eq[i] < 0) continue;
      for (int j = 0; j < 6; ++j) {
        if (eq[j] < eq[i]) continue;
        const double a = A[(i % 3) + 3 * (j % 3)];
        const int* b = &m->cols[m->rowptr[eq[i]]];
        const int* en = &m->cols[0] + m->rowptr[eq[i] + 1];
        const int* f = std::lower_bound(b, en, eq[j]);
        values[f - &m->cols[0]] += (i / 3 == j / 3) ? a : -a;
      }
    }
  }
  return (int)m->cols.size();
}

// K (which 0), M (1) or C (2) of element iel, n x n column-major; returns n * n
extern "C" int oracle_get_element_matrix(OracleModel* m, int iel, int which, double* mat) {
  if (!m || iel < 0 || iel >= (int)m->elems.size()) return 0;
  const Elem& e = m->elems[iel];
  const int nn = e.n * e.n;
  const std::vector<double>& src = which == 0 ? e.K : which == 1 ? e.M : e.C;
  if (which == 2 && !e.hasC) { std::fill(mat, mat + nn, 0.0); return nn; }
  std::copy(src.begin(), src.begin() + nn, mat);
  return nn;
}

// number of DOFs of element iel (6 per triad + generalized DOFs)
extern "C" int oracle_get_element_size(OracleModel* m, int iel) {
  if (!m || iel < 0 || iel >= (int)m->elems.size()) return 0;
  return m->elems[iel].n;
}

// generalized DOF values of element iel (genDOFs%ur); returns their number
extern "C" int oracle_get_gen_dofs(OracleModel* m, int iel, double* v) {
  if (!m || iel < 0 || iel >= (int)m->elems.size()) return 0;
  const Elem& e = m->elems[iel];
  if (v) std::copy(e.genUr.begin(), e.genUr.end(), v);
  return e.nGen;
}

extern "C" int oracle_get_force_vector(OracleModel* m, int which, double* vec) {
  if (!m) return 0;
  const std::vector<double>& v = which == 0 ? m->FSk : which == 1 ? m->FDk : which == 2 ? m->FIk : m->Qk;
  std::copy(v.begin(), v.end(), vec);
  return m->neq;
}
