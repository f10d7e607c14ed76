// sg_oracle.cpp -- CPU FP64 restatement of SPECFEM3D_GEOTECH's serial solve path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it as the
// checker.  The product (the CUDA library under specfem3d_geotech_gb300/) never
// links, loads or calls it.
//
// Parity status: UNPINNED against the reference binary.  The reference is
// Fortran 90 and no Fortran compiler exists on either build machine, and the
// reference ships no tests, golden vectors or stored outputs.  The restatement
// is pinned instead by analytic known answers (GLL tables, rigid-body null
// space of K_e, the confined gravity column, invariants at the Lode corners,
// Mohr-Coulomb hand values) checked in tests/test_oracle_kat.py.
//
// Every routine follows one reference routine with the same loop nesting and
// the same sequential reduction order; the citation (file:line, paths inside
// the reference project) is given on each.  Arrays keep the reference's
// conventions: element dof vectors are node-major [n0x n0y n0z n1x ...],
// global vectors are 0:neq with index 0 the sink of constrained dofs,
// K_e is stored column-major 81x81 per element (k(row,col,e)).
// Node ids are 0-based here (the reference is 1-based); gdof values keep the
// reference meaning (0 = fixed, 1..neq = equation number).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

namespace {

constexpr int NDIM = 3, NGLL = 27, NENOD = 27, NEDOF = 81, NST = 6, NGNODE = 8;
constexpr double ZERO = 0.0, HALF = 0.5, ONE = 1.0, TWO = 2.0;
constexpr double PI = 3.141592653589793;
constexpr double DEG2RAD = PI / 180.0, RAD2DEG = 180.0 / PI;
constexpr double INFTOL = 1.0e32, ZEROTOL = 1.0e-12;

// ---------------------------------------------------------------------------
// Quadrature tables for NGLL = 3 per direction.
// ---------------------------------------------------------------------------
struct Tables {
  double xigll[3], wgll[3];
  double gll_weights[NGLL];
  double gll_points[NDIM][NGLL];
  double lagrange[NGLL][NGLL];          // lagrange_gll(ii,n)
  double dlagrange[NDIM][NGLL][NGLL];   // dlagrange_gll(a,ii,n)
  double dshape[NDIM][NGNODE][NGLL];    // dshape_hex8(a,gnod,igll)
  double shape[NGNODE][NGLL];           // shape_hex8(gnod,i,j,k) flattened
  int hex8_gnode[8];                    // corner local nodes (0-based)
  std::vector<int> face_nodes[6];       // Exodus faces 1..6 -> local nodes
};

// GLL points/weights for 3 points: zwgljd with alpha=beta=0 gives {-1,0,1}
// and {1/3,4/3,1/3} (src/gll_library.f90:717-783); hex2spec forces the middle
// abscissa to exactly zero (src/mesh_spec.f90:67-69).  The closed form is used.
//
// lagrange1dGLL (src/gll_library.f90:257-299): product form for phi and the
// sum-of-products form for its derivative, in the reference's term order.
void lagrange1d(const double* xii, double xi, double* phi, double* dphi) {
  const int n = 3;
  for (int i = 0; i < n; ++i) {
    double term[3], dterm[3];
    int k = 0;
    phi[i] = 1.0;
    for (int j = 0; j < n; ++j) {
      if (j != i) {
        term[k] = (xi - xii[j]) / (xii[i] - xii[j]);
        dterm[k] = 1.0 / (xii[i] - xii[j]);
        ++k;
        phi[i] = phi[i] * (xi - xii[j]) / (xii[i] - xii[j]);
      }
    }
    double sum_term[3] = {1.0, 1.0, 1.0};
    for (int jj = 0; jj < n - 1; ++jj)
      for (int kk = 0; kk < n - 1; ++kk)
        sum_term[jj] = (kk == jj) ? sum_term[jj] * dterm[kk] : sum_term[jj] * term[kk];
    dphi[i] = 0.0;
    for (int jj = 0; jj < n - 1; ++jj) dphi[i] = dphi[i] + sum_term[jj];
  }
}

void build_tables(Tables& T) {
  T.xigll[0] = -1.0; T.xigll[1] = 0.0; T.xigll[2] = 1.0;
  T.wgll[0] = 1.0 / 3.0; T.wgll[1] = 4.0 / 3.0; T.wgll[2] = 1.0 / 3.0;
  // gll_quadrature (src/gll_library.f90:14-82): n runs k (z) slowest, i (x) fastest.
  int n = 0;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        T.gll_points[0][n] = T.xigll[i];
        T.gll_points[1][n] = T.xigll[j];
        T.gll_points[2][n] = T.xigll[k];
        T.gll_weights[n] = T.wgll[i] * T.wgll[j] * T.wgll[k];
        ++n;
      }
  for (int ii = 0; ii < NGLL; ++ii) {
    double lx[3], ldx[3], ly[3], ldy[3], lz[3], ldz[3];
    lagrange1d(T.xigll, T.gll_points[0][ii], lx, ldx);
    lagrange1d(T.xigll, T.gll_points[1][ii], ly, ldy);
    lagrange1d(T.xigll, T.gll_points[2][ii], lz, ldz);
    int m = 0;
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          T.lagrange[ii][m] = lx[i] * ly[j] * lz[k];
          T.dlagrange[0][ii][m] = ldx[i] * ly[j] * lz[k];
          T.dlagrange[1][ii][m] = lx[i] * ldy[j] * lz[k];
          T.dlagrange[2][ii][m] = lx[i] * ly[j] * ldz[k];
          ++m;
        }
  }
  // dshape_function_hex8 (src/shape_library.f90:104-216), Exodus corner order.
  const double e8 = 0.125;
  int igll = 0;
  for (int k = 0; k < 3; ++k) {
    double zp = 1.0 + T.xigll[k], zm = 1.0 - T.xigll[k];
    for (int j = 0; j < 3; ++j) {
      double ep = 1.0 + T.xigll[j], em = 1.0 - T.xigll[j];
      for (int i = 0; i < 3; ++i) {
        double xp = 1.0 + T.xigll[i], xm = 1.0 - T.xigll[i];
        double (*d)[NGNODE][NGLL] = T.dshape;
        d[0][0][igll] = -e8 * em * zm; d[0][1][igll] = e8 * em * zm;
        d[0][2][igll] = e8 * ep * zm;  d[0][3][igll] = -e8 * ep * zm;
        d[0][4][igll] = -e8 * em * zp; d[0][5][igll] = e8 * em * zp;
        d[0][6][igll] = e8 * ep * zp;  d[0][7][igll] = -e8 * ep * zp;
        d[1][0][igll] = -e8 * xm * zm; d[1][1][igll] = -e8 * xp * zm;
        d[1][2][igll] = e8 * xp * zm;  d[1][3][igll] = e8 * xm * zm;
        d[1][4][igll] = -e8 * xm * zp; d[1][5][igll] = -e8 * xp * zp;
        d[1][6][igll] = e8 * xp * zp;  d[1][7][igll] = e8 * xm * zp;
        d[2][0][igll] = -e8 * xm * em; d[2][1][igll] = -e8 * xp * em;
        d[2][2][igll] = -e8 * xp * ep; d[2][3][igll] = -e8 * xm * ep;
        d[2][4][igll] = e8 * xm * em;  d[2][5][igll] = e8 * xp * em;
        d[2][6][igll] = e8 * xp * ep;  d[2][7][igll] = e8 * xm * ep;
        // shape_function_hex8 (src/shape_library.f90:14-98)
        T.shape[0][igll] = e8 * xm * em * zm; T.shape[1][igll] = e8 * xp * em * zm;
        T.shape[2][igll] = e8 * xp * ep * zm; T.shape[3][igll] = e8 * xm * ep * zm;
        T.shape[4][igll] = e8 * xm * em * zp; T.shape[5][igll] = e8 * xp * em * zp;
        T.shape[6][igll] = e8 * xp * ep * zp; T.shape[7][igll] = e8 * xm * ep * zp;
        ++igll;
      }
    }
  }
  // prepare_hex (src/element.f90:21-45): corners 1,3,9,7,19,21,27,25 (1-based).
  const int g[8] = {1, 3, 9, 7, 19, 21, 27, 25};
  for (int a = 0; a < 8; ++a) T.hex8_gnode[a] = g[a] - 1;
  // prepare_hexface (src/element.f90:48-141): 1=y-min 2=x-max 3=y-max 4=x-min 5=z-min 6=z-max.
  for (int f = 0; f < 6; ++f) T.face_nodes[f].clear();
  int inode = 0;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        if (i == 0) T.face_nodes[3].push_back(inode);
        if (i == 2) T.face_nodes[1].push_back(inode);
        if (j == 0) T.face_nodes[0].push_back(inode);
        if (j == 2) T.face_nodes[2].push_back(inode);
        if (k == 0) T.face_nodes[4].push_back(inode);
        if (k == 2) T.face_nodes[5].push_back(inode);
        ++inode;
      }
}

const Tables& tables() {
  static Tables T;
  static bool init = false;
  if (!init) { build_tables(T); init = true; }
  return T;
}

// ---------------------------------------------------------------------------
// Small dense math.
// ---------------------------------------------------------------------------
// compute_cmat (src/elastic.f90:13-42)
void compute_cmat(double E, double v, double c[6][6]) {
  for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) c[i][j] = 0.0;
  double onepv = ONE + v, onemv = ONE - v, onem2v = ONE - TWO * v;
  double Efact = E / (onepv * onem2v);
  c[0][0] = onemv * Efact; c[0][1] = v * Efact; c[0][2] = c[0][1];
  c[1][0] = c[0][1]; c[1][1] = c[0][0]; c[1][2] = c[0][1];
  c[2][0] = c[0][2]; c[2][1] = c[1][2]; c[2][2] = c[0][0];
  c[3][3] = HALF * onem2v * Efact;
  c[4][4] = c[3][3];
  c[5][5] = c[3][3];
}

// compute_bmat (src/preprocess.f90:12-68)
void compute_bmat(const double deriv[3][NENOD], double b[6][NEDOF]) {
  for (int s = 0; s < 6; ++s) for (int j = 0; j < NEDOF; ++j) b[s][j] = 0.0;
  for (int n = 0; n < NENOD; ++n) {
    int j1 = 3 * n, j2 = j1 + 1, j3 = j1 + 2;
    double dx = deriv[0][n], dy = deriv[1][n], dz = deriv[2][n];
    b[0][j1] = dx; b[1][j2] = dy; b[2][j3] = dz;
    b[3][j1] = dy; b[3][j2] = dx;
    b[4][j2] = dz; b[4][j3] = dy;
    b[5][j1] = dz; b[5][j3] = dx;
  }
}

// determinant, 3x3 case (src/math_library.f90:66-85)
double determinant3(const double x[3][3]) {
  double det = x[0][0] * (x[1][1] * x[2][2] - x[2][1] * x[1][2]);
  det = det - x[0][1] * (x[1][0] * x[2][2] - x[2][0] * x[1][2]);
  det = det + x[0][2] * (x[1][0] * x[2][1] - x[2][0] * x[1][1]);
  return det;
}

// invert, 3x3 cofactor case (src/math_library.f90:91-138)
void invert3(double x[3][3]) {
  double det = x[0][0] * (x[1][1] * x[2][2] - x[2][1] * x[1][2]);
  det = det - x[0][1] * (x[1][0] * x[2][2] - x[2][0] * x[1][2]);
  det = det + x[0][2] * (x[1][0] * x[2][1] - x[2][0] * x[1][1]);
  double j11 = x[1][1] * x[2][2] - x[2][1] * x[1][2];
  double j21 = -x[1][0] * x[2][2] + x[2][0] * x[1][2];
  double j31 = x[1][0] * x[2][1] - x[2][0] * x[1][1];
  double j12 = -x[0][1] * x[2][2] + x[2][1] * x[0][2];
  double j22 = x[0][0] * x[2][2] - x[2][0] * x[0][2];
  double j32 = -x[0][0] * x[2][1] + x[2][0] * x[0][1];
  double j13 = x[0][1] * x[1][2] - x[1][1] * x[0][2];
  double j23 = -x[0][0] * x[1][2] + x[1][0] * x[0][2];
  double j33 = x[0][0] * x[1][1] - x[1][0] * x[0][1];
  x[0][0] = j11 / det; x[0][1] = j12 / det; x[0][2] = j13 / det;
  x[1][0] = j21 / det; x[1][1] = j22 / det; x[1][2] = j23 / det;
  x[2][0] = j31 / det; x[2][1] = j32 / det; x[2][2] = j33 / det;
}

// stress_invariant (src/math_library.f90:144-186)
void stress_invariant(const double* s, double& sigm, double& dsbar, double& theta) {
  const double small = 1.e-12, three = 3.0, six = 6.0;
  double sq3 = std::sqrt(three);
  double s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3], s5 = s[4], s6 = s[5];
  sigm = (s1 + s2 + s3) / three;
  double d2 = ((s1 - s2) * (s1 - s2) + (s2 - s3) * (s2 - s3) + (s3 - s1) * (s3 - s1)) / six +
              s4 * s4 + s5 * s5 + s6 * s6;
  if (d2 < small) d2 = small;
  double ds1 = s1 - sigm, ds2 = s2 - sigm, ds3 = s3 - sigm;
  double d3 = ds1 * ds2 * ds3 - ds1 * s5 * s5 - ds2 * s6 * s6 - ds3 * s4 * s4 + TWO * s4 * s5 * s6;
  dsbar = sq3 * std::sqrt(d2);
  if (dsbar < small) {
    theta = 0.0;
  } else {
    double sq = std::sqrt(d2);
    double sine = -three * sq3 * d3 / (TWO * (sq * sq * sq));
    if (sine >= ONE) sine = ONE;
    if (sine < -ONE) sine = -ONE;
    theta = std::asin(sine) / three;
  }
}

// mohcouf (src/plastic_library.f90:95-108); phi in degrees, theta in radians.
double mohcouf(double phi, double c, double sigm, double dsbar, double theta) {
  const double r3 = 3.0;
  double phir = phi * DEG2RAD;
  double snph = std::sin(phir), csph = std::cos(phir);
  double csth = std::cos(theta), snth = std::sin(theta);
  return snph * sigm + dsbar * (csth / std::sqrt(r3) - snth * snph / r3) - c * csph;
}

// mohcouq (src/plastic_library.f90:116-143), corner branch |sin(theta)|>0.49.
void mohcouq(double psi, double dsbar, double theta, double& dq1, double& dq2, double& dq3) {
  const double pt49 = 0.49, pt5 = 0.5, r3 = 3.0;
  double psir = psi * DEG2RAD;
  double snth = std::sin(theta);
  double snps = std::sin(psir);
  double sq3 = std::sqrt(r3);
  dq1 = snps;
  if (std::fabs(snth) > pt49) {
    double c1 = ONE;
    if (snth < ZERO) c1 = -ONE;
    dq2 = (sq3 * pt5 - c1 * snps * pt5 / sq3) * sq3 * pt5 / dsbar;
    dq3 = ZERO;
  } else {
    double csth = std::cos(theta);
    double cs3th = std::cos(r3 * theta);
    double tn3th = std::tan(r3 * theta);
    double tnth = snth / csth;
    dq2 = sq3 * csth / dsbar * ((ONE + tnth * tn3th) + snps * (tn3th - tnth) / sq3) * pt5;
    dq3 = pt5 * r3 * (sq3 * snth + snps * csth) / (cs3th * dsbar * dsbar);
  }
}

// formm (src/plastic_library.f90:150-208)
void formm(const double* st, double m1[6][6], double m2[6][6], double m3[6][6]) {
  const double r3 = 3.0, r6 = 6.0;
  double sx = st[0], sy = st[1], sz = st[2], txy = st[3], tyz = st[4], tzx = st[5];
  double sigm = (sx + sy + sz) / r3;
  double dx = sx - sigm, dy = sy - sigm, dz = sz - sigm;
  for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) { m1[i][j] = 0.0; m2[i][j] = 0.0; m3[i][j] = 0.0; }
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m1[i][j] = ONE / (r3 * sigm);
  for (int i = 0; i < 3; ++i) { m2[i][i] = TWO; m2[i + 3][i + 3] = r6; }
  m2[0][1] = -ONE; m2[0][2] = -ONE; m2[1][2] = -ONE;
  m3[0][0] = dx; m3[0][1] = dz; m3[0][2] = dy; m3[0][3] = txy; m3[0][4] = -TWO * tyz; m3[0][5] = tzx;
  m3[1][1] = dy; m3[1][2] = dx; m3[1][3] = txy; m3[1][4] = tyz; m3[1][5] = -TWO * tzx;
  m3[2][2] = dz; m3[2][3] = -TWO * txy; m3[2][4] = tyz; m3[2][5] = tzx;
  m3[3][3] = -r3 * dz; m3[3][4] = r3 * tzx; m3[3][5] = r3 * tyz;
  m3[4][4] = -r3 * dx; m3[4][5] = r3 * txy;
  m3[5][5] = -r3 * dy;
  for (int i = 0; i < 6; ++i)
    for (int j = i + 1; j < 6; ++j) { m1[j][i] = m1[i][j]; m2[j][i] = m2[i][j]; m3[j][i] = m3[i][j]; }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) { m1[i][j] /= r3; m2[i][j] /= r3; m3[i][j] /= r3; }
}

// dt_viscoplas (src/plastic_library.f90:17-39)
double dt_viscoplas(int nmat, const double* nuf, const double* phif, const double* ymf,
                    const unsigned char* ismat) {
  const double r4 = 4.0;
  double dt_min = INFTOL;
  for (int i = 0; i < nmat; ++i) {
    if (ismat && !ismat[i]) continue;
    double snphi = std::sin(phif[i] * DEG2RAD);
    double dt = r4 * (ONE + nuf[i]) * (ONE - TWO * nuf[i]) /
                (ymf[i] * (ONE - TWO * nuf[i] + snphi * snphi));
    if (dt < dt_min) dt_min = dt;
  }
  return dt_min;
}

// strength_reduction (src/plastic_library.f90:42-88); returns istat.
int strength_reduction(double srf, bool phinu, int nmat, const double* coh, const double* nu,
                       const double* phi, const double* psi, double* cohf, double* nuf,
                       double* phif, double* psif) {
  for (int i = 0; i < nmat; ++i) { cohf[i] = coh[i]; nuf[i] = nu[i]; phif[i] = phi[i]; psif[i] = psi[i]; }
  int istat = 0;
  if (srf != ONE) {
    for (int i = 0; i < nmat; ++i) {
      double tnphi = std::tan(phi[i] * DEG2RAD);
      phif[i] = std::atan(tnphi / srf) * RAD2DEG;
      double tnpsi = std::tan(psi[i] * DEG2RAD);
      psif[i] = std::atan(tnpsi / srf) * RAD2DEG;
      cohf[i] = coh[i] / srf;
    }
  }
  if (!phinu) return istat;
  for (int i = 0; i < nmat; ++i) {
    double omtnu = ONE - TWO * nu[i];
    double snphif = std::sin(phif[i] * DEG2RAD);
    if (snphif < omtnu) {
      double snphi = std::sin(phi[i] * DEG2RAD);
      double beta = snphi / omtnu;
      if (beta < ONE) beta = ONE + ZEROTOL;
      nuf[i] = HALF * (ONE - snphif / beta);
      istat = 1;
    }
  }
  return istat;
}

// ---------------------------------------------------------------------------
// Model: spectral mesh + material blocks + dof numbering.
// ---------------------------------------------------------------------------
struct Model {
  int nnode = 0, nelmt = 0, nmatblk = 0, neq = 0;
  std::vector<double> g_coord;   // 3*nnode
  std::vector<int> g_num;        // 27*nelmt, 0-based nodes
  std::vector<int> mat_id;       // nelmt, 1-based block id
  std::vector<double> gam, ym, nu, phi, coh, psi;
  std::vector<int> gdof;         // 3*nnode
  std::vector<int> gdof_elmt;    // 81*nelmt
  bool iswater = false;          // water table set (water: line)
  std::vector<double> wpressure; // nnode pore pressure
  std::vector<char> submerged;   // nnode
};

// get_global (src/mesh_spec.f90:146-262): lexicographic segmented sort with
// tolerance 1e-10*|xmax-xmin|, one pass per coordinate.  Returns the number of
// unique points; iglob is 1-based like the reference.
int get_global(std::vector<double> xp, std::vector<double> yp, std::vector<double> zp,
               std::vector<int>& iglob, double xmin, double xmax) {
  const size_t np = xp.size();
  std::vector<int> iloc(np);
  std::iota(iloc.begin(), iloc.end(), 0);
  std::vector<char> ifseg(np, 0);
  std::vector<size_t> ninseg;
  ninseg.push_back(np);
  ifseg[0] = 1;
  double smalltol = 1.e-10 * std::fabs(xmax - xmin);
  std::vector<size_t> ind;
  std::vector<int> iw;
  std::vector<double> w;
  for (int j = 0; j < 3; ++j) {
    std::vector<double>& key = (j == 0) ? xp : (j == 1) ? yp : zp;
    size_t ioff = 0;
    for (size_t iseg = 0; iseg < ninseg.size(); ++iseg) {
      size_t n = ninseg[iseg];
      ind.resize(n);
      std::iota(ind.begin(), ind.end(), 0);
      std::stable_sort(ind.begin(), ind.end(),
                       [&](size_t a, size_t b) { return key[ioff + a] < key[ioff + b]; });
      iw.assign(iloc.begin() + ioff, iloc.begin() + ioff + n);
      for (size_t i = 0; i < n; ++i) iloc[ioff + i] = iw[ind[i]];
      for (std::vector<double>* arr : {&xp, &yp, &zp}) {
        w.assign(arr->begin() + ioff, arr->begin() + ioff + n);
        for (size_t i = 0; i < n; ++i) (*arr)[ioff + i] = w[ind[i]];
      }
      ioff += n;
    }
    for (size_t i = 1; i < np; ++i)
      if (std::fabs(key[i] - key[i - 1]) > smalltol) ifseg[i] = 1;
    ninseg.clear();
    for (size_t i = 0; i < np; ++i) {
      if (ifseg[i]) ninseg.push_back(1);
      else ninseg.back() += 1;
    }
  }
  iglob.assign(np, 0);
  int ig = 0;
  for (size_t i = 0; i < np; ++i) {
    if (ifseg[i]) ++ig;
    iglob[iloc[i]] = ig;
  }
  return ig;
}

// hex2spec (src/mesh_spec.f90:17-143) + get_global_indirect_addressing
// (src/mesh_spec.f90:357-386).  conn8 is 1-based Exodus hex8 connectivity.
void hex2spec(Model& M, int nnode8, const double* x8, const double* y8, const double* z8,
              const int* conn8) {
  const Tables& T = tables();
  const int nelmt = M.nelmt;
  double xmin = x8[0], xmax = x8[0];
  for (int i = 0; i < nnode8; ++i) { xmin = std::min(xmin, x8[i]); xmax = std::max(xmax, x8[i]); }
  const size_t npoint = (size_t)nelmt * NGLL;
  std::vector<double> xs(npoint), ys(npoint), zs(npoint);
  size_t ip = 0;
  for (int e = 0; e < nelmt; ++e)
    for (int n = 0; n < NGLL; ++n) {
      double xg = 0, yg = 0, zg = 0;
      for (int g = 0; g < 8; ++g) {
        int nd = conn8[(size_t)e * 8 + g] - 1;
        xg = xg + T.shape[g][n] * x8[nd];
        yg = yg + T.shape[g][n] * y8[nd];
        zg = zg + T.shape[g][n] * z8[nd];
      }
      xs[ip] = xg; ys[ip] = yg; zs[ip] = zg; ++ip;
    }
  std::vector<int> iglob;
  int nn = get_global(xs, ys, zs, iglob, xmin, xmax);
  // first-touch renumbering
  std::vector<int> mask(nn + 1, -1);
  int inumber = 0;
  for (size_t i = 0; i < npoint; ++i) {
    int o = iglob[i];
    if (mask[o] == -1) { ++inumber; mask[o] = inumber; }
    iglob[i] = mask[o];
  }
  M.nnode = nn;
  M.g_coord.assign((size_t)3 * nn, 0.0);
  M.g_num.assign(npoint, 0);
  for (size_t i = 0; i < npoint; ++i) {
    int nd = iglob[i] - 1;
    M.g_num[i] = nd;
    M.g_coord[(size_t)3 * nd + 0] = xs[i];
    M.g_coord[(size_t)3 * nd + 1] = ys[i];
    M.g_coord[(size_t)3 * nd + 2] = zs[i];
  }
}

// apply_bc (src/apply_bc.f90:7-143): zero-valued face constraints, then
// node-major numbering of the free dofs.  bc[d] holds (elem 1-based, face 1..6) pairs.
void apply_bc(Model& M, const std::vector<std::pair<int, int>> bc[3]) {
  const Tables& T = tables();
  M.gdof.assign((size_t)3 * M.nnode, 1);
  for (int d = 0; d < 3; ++d)
    for (auto& ef : bc[d]) {
      int e = ef.first - 1, f = ef.second - 1;
      for (int ln : T.face_nodes[f]) M.gdof[(size_t)3 * M.g_num[(size_t)e * NGLL + ln] + d] = 0;
    }
  int neq = 0;
  for (int j = 0; j < M.nnode; ++j)
    for (int i = 0; i < 3; ++i)
      if (M.gdof[(size_t)3 * j + i] != 0) M.gdof[(size_t)3 * j + i] = ++neq;
  M.neq = neq;
}

// compute_pressure (src/compute_pressure.f90:10-186).  water[m] flags the water
// materials; the water-surface file is read list-directed.  Returns 0, or -1
// with errtag set.
struct WaterSurf {
  int stype = 0, rdir = 1;
  double rx1 = 0, rx2 = 0, z1 = 0, z2 = 0;
  std::vector<int> ielmt, iface;  // 1-based element, face 1..6
};

int compute_pressure(Model& M, const std::vector<char>& water, const std::string& wsfile, std::string& errtag) {
  const Tables& T = tables();
  const double gamw = 9.81;
  errtag = "ERROR: unknown!";
  M.submerged.assign(M.nnode, 0);
  for (int e = 0; e < M.nelmt; ++e)
    if (water[M.mat_id[e] - 1])
      for (int i = 0; i < NGLL; ++i) M.submerged[M.g_num[(size_t)e * NGLL + i]] = 1;
  std::ifstream in(wsfile);
  if (!in) { errtag = "ERROR: input file \"" + wsfile + "\" cannot be opened!"; return -1; }
  std::string all((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  for (char& ch : all) if (ch == ',') ch = ' ';
  std::stringstream ss(all);
  int nwsurf = 0;
  ss >> nwsurf;
  std::vector<WaterSurf> ws(nwsurf);
  for (auto& w : ws) {
    ss >> w.stype;
    if (w.stype == 0) ss >> w.rdir >> w.rx1 >> w.rx2 >> w.z1;
    else if (w.stype == 1) ss >> w.rdir >> w.rx1 >> w.rx2 >> w.z1 >> w.z2;
    else if (w.stype == 2) {
      int nface = 0;
      ss >> nface;
      w.ielmt.resize(nface); w.iface.resize(nface);
      for (int f = 0; f < nface; ++f) ss >> w.ielmt[f] >> w.iface[f];
    }
  }
  M.wpressure.assign(M.nnode, 0.0);
  for (int n = 0; n < M.nnode; ++n) {
    if (!M.submerged[n]) continue;
    const double* xp = &M.g_coord[(size_t)3 * n];
    bool next_node = false;
    for (int w = 0; w < nwsurf && !next_node; ++w) {
      const WaterSurf& S = ws[w];
      if (S.stype == 0) {
        double z = S.z1;
        if (xp[S.rdir - 1] >= S.rx1 && xp[S.rdir - 1] <= S.rx2 && xp[2] <= z) {
          if (z > xp[2]) M.wpressure[n] = gamw * (z - xp[2]);
          next_node = true;
        }
      } else if (S.stype == 1) {
        if (xp[S.rdir - 1] >= std::min(S.rx1, S.rx2) && xp[S.rdir - 1] <= std::max(S.rx1, S.rx2) &&
            xp[2] <= std::max(S.z1, S.z2)) {
          double z = S.z1 + (S.z2 - S.z1) * (xp[S.rdir - 1] - S.rx1) / (S.rx2 - S.rx1);
          if (z > xp[2]) M.wpressure[n] = gamw * (z - xp[2]);
          next_node = true;
        }
      } else if (S.stype == 2) {
        for (size_t f = 0; f < S.ielmt.size() && !next_node; ++f) {
          // face corners hexface(iface)%gnode = node(1), node(3), node(9), node(7)
          const std::vector<int>& fn = T.face_nodes[S.iface[f] - 1];
          const int corner[4] = {fn[0], fn[2], fn[8], fn[6]};
          double xf[3][4];
          for (int k = 0; k < 4; ++k)
            for (int c = 0; c < 3; ++c)
              xf[c][k] = M.g_coord[(size_t)3 * M.g_num[(size_t)(S.ielmt[f] - 1) * NGLL + corner[k]] + c];
          double xmin = std::min(std::min(xf[0][0], xf[0][1]), std::min(xf[0][2], xf[0][3]));
          double xmax = std::max(std::max(xf[0][0], xf[0][1]), std::max(xf[0][2], xf[0][3]));
          double ymin = std::min(std::min(xf[1][0], xf[1][1]), std::min(xf[1][2], xf[1][3]));
          double ymax = std::max(std::max(xf[1][0], xf[1][1]), std::max(xf[1][2], xf[1][3]));
          double zmin = std::min(std::min(xf[2][0], xf[2][1]), std::min(xf[2][2], xf[2][3]));
          double zmax = std::max(std::max(xf[2][0], xf[2][1]), std::max(xf[2][2], xf[2][3]));
          if (!(xp[0] >= xmin && xp[0] <= xmax && xp[1] >= ymin && xp[1] <= ymax && xp[2] <= zmax)) continue;
          double v1[3], v2[3];
          for (int c = 0; c < 3; ++c) { v1[c] = xf[c][1] - xf[c][0]; v2[c] = xf[c][2] - xf[c][0]; }
          double A = v1[1] * v2[2] - v2[1] * v1[2];
          double B = v2[0] * v1[2] - v1[0] * v2[2];
          double C = v1[0] * v2[1] - v2[0] * v1[1];
          double m3[3][3];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) m3[r][c] = xf[r][c];
          double D = determinant3(m3);  // as written in the reference (z = -(Ax+By+D)/C)
          double z;
          if (C == ZERO) {
            std::fprintf(stderr, "WARNING: free surface face is vertical!\n");
            z = zmax;
          } else {
            z = -(A * xp[0] + B * xp[1] + D) / C;
          }
          if (z > zmax || z < zmin) { errtag = "ERROR: free surface cannot be determined!"; return -1; }
          if (z > xp[2]) M.wpressure[n] = gamw * (z - xp[2]);
          next_node = true;
        }
      }
    }
  }
  M.iswater = true;
  return 0;
}

// gdof_elmt = reshape(gdof(:,g_num(:,e)),(/nedof/)) (src/slope.F90:140-144)
void build_gdof_elmt(Model& M) {
  M.gdof_elmt.assign((size_t)NEDOF * M.nelmt, 0);
  for (int e = 0; e < M.nelmt; ++e)
    for (int a = 0; a < NENOD; ++a)
      for (int d = 0; d < 3; ++d)
        M.gdof_elmt[(size_t)e * NEDOF + 3 * a + d] = M.gdof[(size_t)3 * M.g_num[(size_t)e * NGLL + a] + d];
}

// Per-element geometry at GLL point i: jac = dshape(:,:,i)*coord, det, invert,
// deriv = jac^-1 * dlagrange(:,i,:) (src/preprocess.f90:112-118).
struct ElemGeom {
  double coord[NGNODE][3];
};
void elem_coord(const Model& M, const int* gnod, int e, ElemGeom& G) {
  for (int g = 0; g < NGNODE; ++g) {
    int nd = M.g_num[(size_t)e * NGLL + gnod[g]];
    for (int d = 0; d < 3; ++d) G.coord[g][d] = M.g_coord[(size_t)3 * nd + d];
  }
}
void point_deriv(const ElemGeom& G, int i, double& detjac, double deriv[3][NENOD]) {
  const Tables& T = tables();
  double jac[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double s = 0.0;
      for (int g = 0; g < NGNODE; ++g) s = s + T.dshape[a][g][i] * G.coord[g][b];
      jac[a][b] = s;
    }
  detjac = determinant3(jac);
  invert3(jac);
  for (int d = 0; d < 3; ++d)
    for (int n = 0; n < NENOD; ++n) {
      double s = 0.0;
      for (int a = 0; a < 3; ++a) s = s + jac[d][a] * T.dlagrange[a][i][n];
      deriv[d][n] = s;
    }
}

// stiffness_bodyload (src/preprocess.f90:74-148).  storekm is column-major
// 81x81 per element; extload may be null (no body load).  Only the elements in
// `elist` (or all if null) are processed, in list order, storing K_e in slot
// position (intact-element form of src/excavation.F90:494-496).
void stiffness_bodyload(const Model& M, const int* elist, int nel, const double* nuf,
                        double* storekm, double* dprecon, double* extload, bool gravity,
                        bool pseudoeq, double eqkx, double eqky, double eqkz,
                        const int* gdof_elmt) {
  const Tables& T = tables();
  const int neq = M.neq;
  for (size_t i = 0; i < (size_t)NEDOF * NEDOF * nel; ++i) storekm[i] = 0.0;
  for (int i = 0; i <= neq; ++i) dprecon[i] = 0.0;
  static thread_local std::vector<double> km(NEDOF * NEDOF);
  for (int ie = 0; ie < nel; ++ie) {
    int e = elist ? elist[ie] : ie;
    int imat = M.mat_id[e] - 1;
    double cmat[6][6];
    compute_cmat(M.ym[imat], nuf[imat], cmat);
    ElemGeom G;
    elem_coord(M, T.hex8_gnode, e, G);
    const int* egdof = gdof_elmt + (size_t)e * NEDOF;
    std::fill(km.begin(), km.end(), 0.0);
    double eld[NEDOF] = {0}, eqload[NEDOF] = {0};
    int idof = 0;
    for (int i = 0; i < NGLL; ++i) {
      double detjac, deriv[3][NENOD], bmat[6][NEDOF];
      point_deriv(G, i, detjac, deriv);
      compute_bmat(deriv, bmat);
      // btc = transpose(bmat)*cmat (81x6), then btc*bmat (81x81)
      double btc[NEDOF][6];
      for (int r = 0; r < NEDOF; ++r)
        for (int s = 0; s < 6; ++s) {
          double acc = 0.0;
          for (int t = 0; t < 6; ++t) acc = acc + bmat[t][r] * cmat[t][s];
          btc[r][s] = acc;
        }
      for (int c = 0; c < NEDOF; ++c)
        for (int r = 0; r < NEDOF; ++r) {
          double acc = 0.0;
          for (int s = 0; s < 6; ++s) acc = acc + btc[r][s] * bmat[s][c];
          km[(size_t)c * NEDOF + r] = km[(size_t)c * NEDOF + r] + acc * detjac * T.gll_weights[i];
        }
      idof += 3;
      eld[idof - 1] = eld[idof - 1] + detjac * T.gll_weights[i];
    }
    std::memcpy(storekm + (size_t)ie * NEDOF * NEDOF, km.data(), sizeof(double) * NEDOF * NEDOF);
    for (int k = 0; k < NEDOF; ++k) dprecon[egdof[k]] = dprecon[egdof[k]] + km[(size_t)k * NEDOF + k];
    if (!extload) continue;
    double gm = M.gam[imat];
    if (gravity) {
      // extload(egdof)=extload(egdof)-eld*gam: vector-subscript assignment,
      // right-hand side evaluated before the store.
      double tmp[NEDOF];
      for (int k = 0; k < NEDOF; ++k) tmp[k] = extload[egdof[k]] - eld[k] * gm;
      for (int k = 0; k < NEDOF; ++k) extload[egdof[k]] = tmp[k];
    }
    if (pseudoeq) {
      for (int a = 0; a < NENOD; ++a) {
        eqload[3 * a + 0] = eqkx * eld[3 * a + 2];
        eqload[3 * a + 1] = eqky * eld[3 * a + 2];
        eqload[3 * a + 2] = eqkz * eld[3 * a + 2];
      }
      double tmp[NEDOF];
      for (int k = 0; k < NEDOF; ++k) tmp[k] = extload[egdof[k]] + eqload[k] * gm;
      for (int k = 0; k < NEDOF; ++k) extload[egdof[k]] = tmp[k];
    }
  }
  dprecon[0] = 0.0;
  if (extload) extload[0] = 0.0;
}

// EBE apply kp = sum_e P_e^T K_e P_e p with kp(0)=0 (src/solver.f90:53-59).
void ebe_apply(int neq, int nelmt, const double* k, const double* p, const int* gdof_elmt,
               double* kp) {
  for (int i = 0; i <= neq; ++i) kp[i] = 0.0;
  double y[NEDOF], pe[NEDOF];
  for (int e = 0; e < nelmt; ++e) {
    const int* eg = gdof_elmt + (size_t)e * NEDOF;
    const double* km = k + (size_t)e * NEDOF * NEDOF;
    for (int j = 0; j < NEDOF; ++j) pe[j] = p[eg[j]];
    for (int r = 0; r < NEDOF; ++r) y[r] = 0.0;
    for (int c = 0; c < NEDOF; ++c) {
      double pc = pe[c];
      const double* col = km + (size_t)c * NEDOF;
      for (int r = 0; r < NEDOF; ++r) y[r] = y[r] + col[r] * pc;
    }
    double tmp[NEDOF];
    for (int r = 0; r < NEDOF; ++r) tmp[r] = kp[eg[r]] + y[r];
    for (int r = 0; r < NEDOF; ++r) kp[eg[r]] = tmp[r];
  }
  kp[0] = 0.0;
}

double maxabs(const double* v, int n1) {
  double m = 0.0;
  for (int i = 0; i < n1; ++i) m = std::max(m, std::fabs(v[i]));
  return m;
}
// Dot-product summation order: 0 = sequential (the reference's dot_product),
// 1 = pairwise halving, 2 = 13 interleaved partial sums (a strided split like
// a GPU grid-stride loop), 3 = reverse sequential, 100 + m = m interleaved
// partial sums.  Orders other than 0 exist only to measure how far rounding
// alone moves a solve or a trial (the parity noise floor); they are never the
// default.
int g_dot_order = 0;
double dot_pairwise(const double* a, const double* b, int n) {
  if (n <= 8) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
    return s;
  }
  int h = n / 2;
  return dot_pairwise(a, b, h) + dot_pairwise(a + h, b + h, n - h);
}
double dot(const double* a, const double* b, int n1) {
  if (g_dot_order == 1) return dot_pairwise(a, b, n1);
  if (g_dot_order == 2 || g_dot_order >= 100) {
    // m interleaved partial sums (order 2: m = 13; order 100 + m: m in 1..256)
    const int m = g_dot_order == 2 ? 13 : std::min(256, std::max(1, g_dot_order - 100));
    double part[256] = {0.0};
    for (int i = 0; i < n1; ++i) part[i % m] = part[i % m] + a[i] * b[i];
    double s = 0.0;
    for (int k = 0; k < m; ++k) s = s + part[k];
    return s;
  }
  if (g_dot_order == 3) {
    double s = 0.0;
    for (int i = n1 - 1; i >= 0; --i) s = s + a[i] * b[i];
    return s;
  }
  double s = 0.0;
  for (int i = 0; i < n1; ++i) s = s + a[i] * b[i];
  return s;
}

// pcg_solver (src/solver.f90:14-79).  Returns errcode (0 ok, -1 no convergence).
int pcg_solver(int neq, int nelmt, const double* k, double* u, const double* f,
               const double* dprecon, const int* gdof_elmt, int cg_maxiter, double cg_tol,
               int* cg_iter_out) {
  const int n1 = neq + 1;
  std::vector<double> kp(n1, 0.0), p(n1), r(n1), z(n1);
  if (maxabs(u, n1) > ZERO) ebe_apply(neq, nelmt, k, u, gdof_elmt, kp.data());
  for (int i = 0; i < n1; ++i) { r[i] = f[i] - kp[i]; z[i] = dprecon[i] * r[i]; p[i] = z[i]; }
  int cg_iter;
  for (cg_iter = 1; cg_iter <= cg_maxiter; ++cg_iter) {
    ebe_apply(neq, nelmt, k, p.data(), gdof_elmt, kp.data());
    double rz = dot(r.data(), z.data(), n1);
    double alpha = rz / dot(p.data(), kp.data(), n1);
    for (int i = 0; i < n1; ++i) u[i] = u[i] + alpha * p[i];
    if (std::fabs(alpha) * maxabs(p.data(), n1) / maxabs(u, n1) <= cg_tol) {
      *cg_iter_out = cg_iter;
      return 0;
    }
    for (int i = 0; i < n1; ++i) { r[i] = r[i] - alpha * kp[i]; z[i] = dprecon[i] * r[i]; }
    double beta = dot(r.data(), z.data(), n1) / rz;
    for (int i = 0; i < n1; ++i) p[i] = z[i] + beta * p[i];
  }
  *cg_iter_out = cg_maxiter + 1;  // Fortran DO variable after normal completion
  return -1;
}

// pcg_solver (src/solver.f90:14-79) evaluated in the order the GPU drop-in
// evaluates it, to show that its FP64 kernels differ from the sequential
// restatement above only by evaluation order.  Same algorithm, same
// iterates; what changes:
//  * products are fused multiply-adds, y = fma(K(r,c), p(c), y) for c = 0..80
//    per element row, u = fma(alpha, p, u), r = fma(-alpha, kp, r),
//    p = fma(beta, p, z), dot terms s = fma(a, b, s);
//  * kp(dof) sums its element contributions in element order from zero (the
//    reference's order) but node by node;
//  * the dots are grid-shaped: per-thread partials over a grid-stride loop
//    (r.z over rows 0..neq; p.kp over nodes keyed by their smallest free dof),
//    a 32-lane xor butterfly per warp, the 8 warps of a block in order, and
//    the block partials summed by 256 threads in a strided order, then those
//    256 sums in order.  Grids: rows with ceil(n1/1024) blocks, nodes with
//    ceil(nodes/512) blocks, each capped at 608 (they depend only on the size).
// A checker only: it restates the device code's order so that a test can ask
// for agreement far below the rounding noise of reordering (1e-12, not 1e-8).
namespace gpuorder {
constexpr int NT = 256, NW = 8, NPART_CAP = 608;
int red_grid(long items, long per) {
  long g = (items + per - 1) / per;
  return (int)std::max<long>(1, std::min<long>(g, NPART_CAP));
}
// xor butterfly of 32 lane values; returns lane 0's result
double warp_sum(double v[32]) {
  for (int o = 16; o >= 1; o >>= 1) {
    double w[32];
    for (int l = 0; l < 32; ++l) w[l] = v[l] + v[l ^ o];
    for (int l = 0; l < 32; ++l) v[l] = w[l];
  }
  return v[0];
}
// block partial from the 256 per-thread partials th[b*256 .. b*256+255]
double block_sum(const double* th) {
  double s = 0.0;
  for (int w = 0; w < NW; ++w) {
    double v[32];
    for (int l = 0; l < 32; ++l) v[l] = th[w * 32 + l];
    s = s + warp_sum(v);
  }
  return s;
}
// last-block sum of `grid` partials (one quantity per block, stride nq in
// part, offset q; the thread of index t takes entries t, t+256, ... of the
// interleaved array of grid*nq values, and only threads with t % nq == q
// hold quantity q)
double last_block(const std::vector<double>& part, int grid, int nq, int q) {
  double sfin[NT];
  for (int t = 0; t < NT; ++t) {
    double v = 0.0;
    for (int idx = t; idx < grid * nq; idx += NT) v = v + part[idx];
    sfin[t] = v;
  }
  double s = 0.0;
  for (int t = q; t < NT; t += nq) s = s + sfin[t];
  return s;
}
}  // namespace gpuorder

int pcg_solver_gpu_order(int neq, int nelmt, const double* k, double* u, const double* f, const double* dprecon,
                         const int* gdof_elmt, int cg_maxiter, double cg_tol, int* cg_iter_out) {
  using namespace gpuorder;
  const int n1 = neq + 1;
  const size_t nslots = (size_t)nelmt * NGLL;
  // nodes keyed by their smallest free dof, in increasing key order; each
  // lists its element slots in element order
  std::vector<int> key(nslots), cnt(n1 + 1, 0);
  for (size_t s = 0; s < nslots; ++s) {
    const int* g = gdof_elmt + 3 * s;
    int kk = 0;
    for (int d = 0; d < 3; ++d)
      if (g[d] > 0 && (kk == 0 || g[d] < kk)) kk = g[d];
    key[s] = kk;
    if (kk) cnt[kk]++;
  }
  std::vector<int> gid(n1 + 1, -1);
  int ng = 0;
  for (int kk = 1; kk <= neq; ++kk)
    if (cnt[kk]) gid[kk] = ng++;
  std::vector<int> gptr(ng + 1, 0), gdof(3 * (size_t)ng, 0);
  for (int kk = 1; kk <= neq; ++kk)
    if (cnt[kk]) gptr[gid[kk] + 1] = cnt[kk];
  for (int g = 0; g < ng; ++g) gptr[g + 1] += gptr[g];
  std::vector<int> gent(gptr[ng]), fill(gptr.begin(), gptr.end() - 1);
  for (size_t s = 0; s < nslots; ++s) {
    if (!key[s]) continue;
    const int g = gid[key[s]];
    gent[fill[g]++] = (int)s;
    for (int d = 0; d < 3; ++d) gdof[3 * (size_t)g + d] = gdof_elmt[3 * s + d];
  }
  std::vector<double> Y(nslots * 3), kp(n1, 0.0), p(n1, 0.0), r(n1), z(n1);
  // element products of p_e = fma(beta, pold_e, z_e) (combine) or of v_e
  auto apply = [&](const double* v, bool combine, double beta) {
    for (int e = 0; e < nelmt; ++e) {
      const int* eg = gdof_elmt + (size_t)e * NEDOF;
      const double* km = k + (size_t)e * NEDOF * NEDOF;
      double pe[NEDOF];
      for (int c = 0; c < NEDOF; ++c) pe[c] = combine ? std::fma(beta, v[eg[c]], z[eg[c]]) : v[eg[c]];
      for (int rr = 0; rr < NEDOF; ++rr) {
        double y = 0.0;
        for (int c = 0; c < NEDOF; ++c) y = std::fma(km[(size_t)c * NEDOF + rr], pe[c], y);
        Y[(size_t)e * NEDOF + rr] = y;
      }
    }
  };
  const int ggrid = red_grid(ng, NT * 2), ugrid = red_grid(n1, NT * 4);
  std::vector<double> th((size_t)std::max(ggrid, ugrid) * NT), part(std::max(ggrid, ugrid) * 4);
  // gather kp (and, in an iteration, p = fma(beta, p, z) and the p.kp dot)
  auto gather = [&](bool iter, double beta) -> double {
    std::fill(th.begin(), th.end(), 0.0);
    const long wstride = (long)ggrid * NW * 32;
    for (int g = 0; g < ng; ++g) {
      const int lane = g % 32;
      const long W = ((long)(g / 32)) % ((long)ggrid * NW);
      const long t = W * 32 + lane;  // block W/8, warp W%8
      (void)wstride;
      for (int d = 0; d < 3; ++d) {
        double acc = 0.0;
        for (int sl = gptr[g]; sl < gptr[g + 1]; ++sl) acc = acc + Y[(size_t)gent[sl] * 3 + d];
        const int gd = gdof[3 * (size_t)g + d];
        if (!gd) continue;
        kp[gd] = acc;
        if (iter) {
          p[gd] = std::fma(beta, p[gd], z[gd]);
          th[t] = std::fma(p[gd], acc, th[t]);
        }
      }
    }
    if (!iter) return 0.0;
    for (int b = 0; b < ggrid; ++b) part[b] = block_sum(th.data() + (size_t)b * NT);
    return last_block(part, ggrid, 1, 0);
  };
  // update: u, r, z and the r.z dot (init: r = f - kp, z = D r)
  double maxp = 0.0, maxu = 0.0;
  auto update = [&](bool init, double alpha) -> double {
    std::fill(th.begin(), th.end(), 0.0);
    const long S = (long)ugrid * NT;
    maxp = 0.0; maxu = 0.0;
    for (long i = 0; i < n1; ++i) {
      const long t = i % S;
      if (init) {
        r[i] = f[i] - kp[i];
        z[i] = dprecon[i] * r[i];
      } else {
        u[i] = std::fma(alpha, p[i], u[i]);
        r[i] = std::fma(-alpha, kp[i], r[i]);
        z[i] = dprecon[i] * r[i];
        maxp = std::max(maxp, std::fabs(p[i]));
        maxu = std::max(maxu, std::fabs(u[i]));
      }
      th[t] = std::fma(r[i], z[i], th[t]);
    }
    for (int b = 0; b < ugrid; ++b) {
      part[(size_t)b * 4 + 0] = part[(size_t)b * 4 + 1] = part[(size_t)b * 4 + 3] = 0.0;
      part[(size_t)b * 4 + 2] = block_sum(th.data() + (size_t)b * NT);
    }
    return last_block(part, ugrid, 4, 2);
  };
  apply(u, false, 0.0);
  gather(false, 0.0);
  double rz = update(true, 0.0), beta = 0.0;
  for (int it = 1; it <= cg_maxiter; ++it) {
    apply(p.data(), true, beta);
    const double alpha = rz / gather(true, beta);
    const double s = update(false, alpha);
    if (std::fabs(alpha) * maxp / maxu <= cg_tol) {
      *cg_iter_out = it;
      return 0;
    }
    beta = s / rz;
    rz = s;
  }
  *cg_iter_out = cg_maxiter + 1;
  return -1;
}

// One pass of the per-element / per-GLL-point stress, yield, flow and body-load
// block inlined in slope3d (src/slope.F90:311-383) and excavation3d
// (src/excavation.F90:546-616).  `finalize` = (nl_isconv .or. nl_iter==nl_maxiter).
// vmeps/scf are accumulated only when the pointers are non-null (excavation form).
double stress_update(const Model& M, const int* elist, int nel, const double* x,
                     const int* gdof_elmt, const double* ymf, const double* nuf,
                     const double* phif, const double* cohf, const double* psif, double dt,
                     bool nl_isconv, bool finalize, double* evpt, double* stress_elmt,
                     double* bodyload, double* vmeps, double* scf, bool wp_first = false) {
  const Tables& T = tables();
  double fmax = 0.0;
  const double r3 = 3.0, two_third = TWO / r3;
  for (int ie = 0; ie < nel; ++ie) {
    int e = elist ? elist[ie] : ie;
    int imat = M.mat_id[e] - 1;
    double cmat[6][6];
    compute_cmat(ymf[imat], nuf[imat], cmat);
    ElemGeom G;
    elem_coord(M, T.hex8_gnode, e, G);
    const int* egdof = gdof_elmt + (size_t)e * NEDOF;
    double eld[NEDOF], bload[NEDOF];
    for (int j = 0; j < NEDOF; ++j) { eld[j] = x[egdof[j]]; bload[j] = 0.0; }
    for (int i = 0; i < NGLL; ++i) {
      double detjac, deriv[3][NENOD], bmat[6][NEDOF];
      point_deriv(G, i, detjac, deriv);
      compute_bmat(deriv, bmat);
      double eps[6], sigma[6], eff[6];
      double* ev = evpt + ((size_t)e * NGLL + i) * NST;
      double* se = stress_elmt + ((size_t)e * NGLL + i) * NST;
      for (int s = 0; s < 6; ++s) {
        double acc = 0.0;
        for (int j = 0; j < NEDOF; ++j) acc = acc + bmat[s][j] * eld[j];
        eps[s] = acc - ev[s];
      }
      for (int s = 0; s < 6; ++s) {
        double acc = 0.0;
        for (int t = 0; t < 6; ++t) acc = acc + cmat[s][t] * eps[t];
        sigma[s] = acc;
      }
      // effective stress: slope3d adds the pore pressure of submerged nodes
      // after the stored stress (src/slope.F90:334-341), excavation3d before it
      // (src/excavation.F90:566-576)
      const int nd_i = M.g_num[(size_t)e * NGLL + i];
      const bool wet = M.iswater && M.submerged[nd_i];
      if (wp_first) {
        for (int s = 0; s < 6; ++s) eff[s] = sigma[s];
        if (wet)
          for (int s = 0; s < 3; ++s) eff[s] = eff[s] + M.wpressure[nd_i];
        for (int s = 0; s < 6; ++s) eff[s] = eff[s] + se[s];
      } else {
        for (int s = 0; s < 6; ++s) eff[s] = sigma[s] + se[s];
        if (wet)
          for (int s = 0; s < 3; ++s) eff[s] = eff[s] + M.wpressure[nd_i];
      }
      double sigm, dsbar, theta;
      stress_invariant(eff, sigm, dsbar, theta);
      double f = mohcouf(phif[imat], cohf[imat], sigm, dsbar, theta);
      if (f > fmax) fmax = f;
      if (f >= ZERO) {
        double dq1, dq2, dq3, m1[6][6], m2[6][6], m3[6][6], flow[6][6], erate[6], evp[6], devp[6];
        mohcouq(psif[imat], dsbar, theta, dq1, dq2, dq3);
        formm(eff, m1, m2, m3);
        for (int a = 0; a < 6; ++a)
          for (int b = 0; b < 6; ++b) flow[a][b] = f * (m1[a][b] * dq1 + m2[a][b] * dq2 + m3[a][b] * dq3);
        for (int a = 0; a < 6; ++a) {
          double acc = 0.0;
          for (int b = 0; b < 6; ++b) acc = acc + flow[a][b] * eff[b];
          erate[a] = acc;
        }
        for (int a = 0; a < 6; ++a) { evp[a] = erate[a] * dt; ev[a] = ev[a] + evp[a]; }
        for (int a = 0; a < 6; ++a) {
          double acc = 0.0;
          for (int b = 0; b < 6; ++b) acc = acc + cmat[a][b] * evp[b];
          devp[a] = acc;
        }
        if (!nl_isconv && !finalize) {
          double w = detjac * T.gll_weights[i];
          for (int j = 0; j < NEDOF; ++j) {
            double acc = 0.0;
            for (int s = 0; s < 6; ++s) acc = acc + devp[s] * bmat[s][j];
            bload[j] = bload[j] + acc * detjac * T.gll_weights[i];
          }
          (void)w;
        }
      }
      if (finalize) {
        int nd = M.g_num[(size_t)e * NGLL + i];
        if (vmeps) vmeps[nd] = vmeps[nd] + std::sqrt(two_third * (ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2] +
                                                              ev[3] * ev[3] + ev[4] * ev[4] + ev[5] * ev[5]));
        for (int s = 0; s < 6; ++s) se[s] = eff[s];
        if (scf) {
          double phr = phif[imat] * DEG2RAD;
          double sf = (sigm * std::sin(phr) - cohf[imat] * std::cos(phr)) /
                      (-dsbar * (std::cos(theta) / std::sqrt(r3) - std::sin(theta) * std::sin(phr) / r3));
          if (sf < scf[nd]) scf[nd] = sf;
        }
      }
    }
    if (finalize) continue;
    double tmp[NEDOF];
    for (int j = 0; j < NEDOF; ++j) tmp[j] = bodyload[egdof[j]] + bload[j];
    for (int j = 0; j < NEDOF; ++j) bodyload[egdof[j]] = tmp[j];
  }
  bodyload[0] = 0.0;
  return fmax;
}

// elastic_stress (src/postprocess.f90:40-79): sigma = C*B*x per GLL point.
void elastic_stress(const Model& M, const int* gdof_elmt, const double* ymv, const double* nuv,
                    const double* x, double* stress_elmt) {
  const Tables& T = tables();
  for (int e = 0; e < M.nelmt; ++e) {
    int imat = M.mat_id[e] - 1;
    double cmat[6][6];
    compute_cmat(ymv[imat], nuv[imat], cmat);
    ElemGeom G;
    elem_coord(M, T.hex8_gnode, e, G);
    const int* eg = gdof_elmt + (size_t)e * NEDOF;
    double eld[NEDOF];
    for (int j = 0; j < NEDOF; ++j) eld[j] = x[eg[j]];
    for (int i = 0; i < NGLL; ++i) {
      double detjac, deriv[3][NENOD], bmat[6][NEDOF], eps[6];
      point_deriv(G, i, detjac, deriv);
      compute_bmat(deriv, bmat);
      for (int s = 0; s < 6; ++s) {
        double acc = 0.0;
        for (int j = 0; j < NEDOF; ++j) acc = acc + bmat[s][j] * eld[j];
        eps[s] = acc;
      }
      for (int s = 0; s < 6; ++s) {
        double acc = 0.0;
        for (int t = 0; t < 6; ++t) acc = acc + cmat[s][t] * eps[t];
        stress_elmt[((size_t)e * NGLL + i) * NST + s] = acc;
      }
    }
  }
}

// overburden_stress (src/postprocess.f90:10-33)
void overburden_stress(const Model& M, double z0, double p0, double k0, double* stress_elmt) {
  for (int e = 0; e < M.nelmt; ++e) {
    int imat = M.mat_id[e] - 1;
    for (int i = 0; i < NGLL; ++i) {
      double z = M.g_coord[(size_t)3 * M.g_num[(size_t)e * NGLL + i] + 2];
      double szz = p0 - M.gam[imat] * std::fabs(z - z0);
      double* s = stress_elmt + ((size_t)e * NGLL + i) * NST;
      s[2] = szz; s[0] = k0 * szz; s[1] = k0 * szz;
    }
  }
}

// ---------------------------------------------------------------------------
// slope3d (src/slope.F90:13-450), one SRF trial at a time.
// ---------------------------------------------------------------------------
struct TrialResult {
  double srf = 0;
  int cg_tot = 0, nl_iter = 0;
  int converged = 0;   // nl_isconv at exit
  int failed = 0;      // nl_iter == nl_maxiter (the SRF loop exit test, src/slope.F90:441)
  double uxmax = 0, umax = 0, fmax = 0, uerr = 0;
  int errcode = 0;
};

struct SlopeState {
  std::vector<double> storekm, dprecon, extload, bodyload, load, x, oldx, evpt, stress;
  std::vector<int> nl_cg_log;  // cg iterations per NL iteration of the last trial
  std::vector<double> uerr_log;  // uerr per NL iteration of the last trial
};

struct Control {
  double cg_tol = 1e-8, nl_tol = 1e-4;
  int cg_maxiter = 5000, nl_maxiter = 2000;
  int phinu = 0, allelastic = 0, iseqload = 0;
  double eqkx = 0, eqky = 0, eqkz = 0;
};

void slope_setup(const Model& M, const Control& C, SlopeState& S) {
  const int n1 = M.neq + 1;
  S.storekm.assign((size_t)NEDOF * NEDOF * M.nelmt, 0.0);
  S.dprecon.assign(n1, 0.0);
  S.extload.assign(n1, 0.0);
  stiffness_bodyload(M, nullptr, M.nelmt, M.nu.data(), S.storekm.data(), S.dprecon.data(),
                     S.extload.data(), true, C.iseqload != 0, C.eqkx, C.eqky, C.eqkz,
                     M.gdof_elmt.data());
  for (int i = 1; i < n1; ++i) S.dprecon[i] = ONE / S.dprecon[i];
  S.dprecon[0] = 0.0;
}

TrialResult slope_trial(const Model& M, const Control& C, SlopeState& S, double srf) {
  TrialResult R;
  R.srf = srf;
  const int n1 = M.neq + 1, nm = M.nmatblk;
  std::vector<double> cohf(nm), nuf(nm), phif(nm), psif(nm);
  int istat = strength_reduction(srf, C.phinu != 0, nm, M.coh.data(), M.nu.data(), M.phi.data(),
                                 M.psi.data(), cohf.data(), nuf.data(), phif.data(), psif.data());
  double dt = dt_viscoplas(nm, nuf.data(), phif.data(), M.ym.data(), nullptr);
  if (istat == 1) {
    stiffness_bodyload(M, nullptr, M.nelmt, nuf.data(), S.storekm.data(), S.dprecon.data(), nullptr,
                       false, false, 0, 0, 0, M.gdof_elmt.data());
    for (int i = 1; i < n1; ++i) S.dprecon[i] = ONE / S.dprecon[i];
    S.dprecon[0] = 0.0;
  }
  S.stress.assign((size_t)NST * NGLL * M.nelmt, 0.0);
  S.evpt.assign((size_t)NST * NGLL * M.nelmt, 0.0);
  S.bodyload.assign(n1, 0.0);
  S.x.assign(n1, 0.0);
  S.oldx.assign(n1, 0.0);
  S.load.assign(n1, 0.0);
  S.nl_cg_log.clear();
  S.uerr_log.clear();
  int nl_iter = 1;
  bool nl_isconv = false;
  double fmax = 0, uerr = 0;
  for (nl_iter = 1; nl_iter <= C.nl_maxiter; ++nl_iter) {
    fmax = 0.0;
    for (int i = 0; i < n1; ++i) S.load[i] = S.extload[i] + S.bodyload[i];
    S.load[0] = 0.0;
    int cg_iter = 0;
    int err = pcg_solver(M.neq, M.nelmt, S.storekm.data(), S.x.data(), S.load.data(), S.dprecon.data(),
                         M.gdof_elmt.data(), C.cg_maxiter, C.cg_tol, &cg_iter);
    S.nl_cg_log.push_back(cg_iter);
    S.uerr_log.push_back(0.0);
    if (err != 0) { R.errcode = err; R.nl_iter = nl_iter; return R; }
    R.cg_tot += cg_iter;
    S.x[0] = 0.0;
    if (C.allelastic) {
      elastic_stress(M, M.gdof_elmt.data(), M.ym.data(), M.nu.data(), S.x.data(), S.stress.data());
      break;
    }
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n1; ++i) { num = std::max(num, std::fabs(S.x[i] - S.oldx[i])); den = std::max(den, std::fabs(S.x[i])); }
    uerr = num / den;
    S.uerr_log.back() = uerr;
    S.oldx = S.x;
    nl_isconv = uerr <= C.nl_tol;
    bool finalize = nl_isconv || nl_iter == C.nl_maxiter;
    fmax = stress_update(M, nullptr, M.nelmt, S.x.data(), M.gdof_elmt.data(), M.ym.data(), nuf.data(),
                         phif.data(), cohf.data(), psif.data(), dt, nl_isconv, finalize, S.evpt.data(),
                         S.stress.data(), S.bodyload.data(), nullptr, nullptr);
    if (finalize) break;
  }
  if (nl_iter > C.nl_maxiter) nl_iter = C.nl_maxiter;  // not reachable: the loop exits at nl_maxiter
  R.nl_iter = nl_iter;
  R.converged = nl_isconv ? 1 : 0;
  R.failed = (nl_iter == C.nl_maxiter) ? 1 : 0;
  R.fmax = fmax;
  R.uerr = uerr;
  // nodal displacement and summary maxima (src/slope.F90:400-415)
  double uxmax = 0.0, umax = 0.0;
  for (int j = 0; j < M.nnode; ++j) {
    double u[3];
    for (int i = 0; i < 3; ++i) {
      int g = M.gdof[(size_t)3 * j + i];
      u[i] = g ? S.x[g] : 0.0;
      uxmax = std::max(uxmax, std::fabs(u[i]));
    }
    umax = std::max(umax, std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
  }
  R.uxmax = uxmax;
  R.umax = umax;
  return R;
}

// ---------------------------------------------------------------------------
// Deck reader (subset of src/read_input.f90:13-619 and src/apply_bc.f90).
// ---------------------------------------------------------------------------
std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  return s.substr(a, b - a + 1);
}
std::string unquote(std::string v) {
  v = trim(v);
  if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"')) v = v.substr(1, v.size() - 2);
  return v;
}

struct Deck {
  std::map<std::string, std::map<std::string, std::string>> lines;
  std::string dir;
};

bool read_deck(const std::string& path, Deck& D) {
  std::ifstream in(path);
  if (!in) return false;
  size_t sl = path.find_last_of('/');
  D.dir = (sl == std::string::npos) ? "." : path.substr(0, sl);
  std::string line;
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    std::string tag = t;
    while (!tag.empty() && tag.back() == '&') {
      tag.pop_back();
      std::string nx;
      if (!std::getline(in, nx)) return false;
      tag += trim(nx);
    }
    size_t sp = tag.find(' ');
    std::string token = tag.substr(0, sp);
    std::string rest = (sp == std::string::npos) ? "" : tag.substr(sp + 1);
    auto& kv = D.lines[token];
    std::stringstream ss(rest);
    std::string arg;
    while (std::getline(ss, arg, ',')) {
      size_t eq = arg.find('=');
      if (eq == std::string::npos) continue;
      kv[trim(arg.substr(0, eq))] = unquote(arg.substr(eq + 1));
    }
  }
  return true;
}

}  // namespace

// ===========================================================================
// C ABI used by the ctypes wrapper in oracle/pyoracle.py.
// ===========================================================================
extern "C" {

struct OrcModel {
  Model M;
  Control C;
  SlopeState S;
  bool setup_done = false;
  std::vector<double> srf_list;
  std::string err;
};

void* orc_model_from_hex8(int nnode8, const double* x8, const double* y8, const double* z8,
                          int nelmt, const int* conn8, const int* mat_id, int nmatblk,
                          const double* props /* nmatblk x [gam ym nu phi coh psi] */,
                          const int* bc_counts /* 3 */, const int* bc_pairs /* (elem,face) */) {
  OrcModel* h = new OrcModel();
  Model& M = h->M;
  M.nelmt = nelmt;
  hex2spec(M, nnode8, x8, y8, z8, conn8);
  M.mat_id.assign(mat_id, mat_id + nelmt);
  M.nmatblk = nmatblk;
  M.gam.resize(nmatblk); M.ym.resize(nmatblk); M.nu.resize(nmatblk);
  M.phi.resize(nmatblk); M.coh.resize(nmatblk); M.psi.resize(nmatblk);
  for (int i = 0; i < nmatblk; ++i) {
    M.gam[i] = props[6 * i + 0]; M.ym[i] = props[6 * i + 1]; M.nu[i] = props[6 * i + 2];
    M.phi[i] = props[6 * i + 3]; M.coh[i] = props[6 * i + 4]; M.psi[i] = props[6 * i + 5];
  }
  std::vector<std::pair<int, int>> bc[3];
  size_t off = 0;
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < bc_counts[d]; ++i, ++off) bc[d].push_back({bc_pairs[2 * off], bc_pairs[2 * off + 1]});
  apply_bc(M, bc);
  build_gdof_elmt(M);
  return h;
}

// Reads a .sem deck (serial form): preinfo/mesh/bc/material/control lines.
void* orc_model_from_deck(const char* path) {
  Deck D;
  if (!read_deck(path, D)) return nullptr;
  std::string inp = D.lines["preinfo:"].count("inp_path") ? D.lines["preinfo:"]["inp_path"] : "./input";
  // Resolve inp_path relative to the deck's parent directory (decks live in input/).
  std::string base = D.dir + "/";
  auto rd = [&](const std::string& key, const std::string& line) { return base + D.lines[line][key]; };
  std::vector<double> xyz[3];
  const char* keys[3] = {"xfile", "yfile", "zfile"};
  int nnode8 = 0;
  for (int d = 0; d < 3; ++d) {
    std::ifstream f(rd(keys[d], "mesh:"));
    if (!f) return nullptr;
    f >> nnode8;
    xyz[d].resize(nnode8);
    for (int i = 0; i < nnode8; ++i) f >> xyz[d][i];
  }
  std::ifstream fc(rd("confile", "mesh:"));
  int nelmt = 0;
  fc >> nelmt;
  std::vector<int> conn((size_t)8 * nelmt);
  for (auto& c : conn) fc >> c;
  std::ifstream fi(rd("idfile", "mesh:"));
  int ne2;
  fi >> ne2;
  std::vector<int> mid(nelmt);
  for (auto& m : mid) fi >> m;
  std::ifstream fm(base + D.lines["material:"]["matfile"]);
  std::string hdr;
  std::getline(fm, hdr);
  int nmat = 0;
  {
    std::string l;
    std::getline(fm, l);
    nmat = std::atoi(trim(l).c_str());
  }
  std::vector<double> props((size_t)6 * nmat);
  for (int i = 0; i < nmat; ++i) {
    std::string l;
    std::getline(fm, l);
    for (char& ch : l) if (ch == ',') ch = ' ';
    std::stringstream ss(l);
    int id, dom, typ;
    ss >> id >> dom >> typ;
    for (int k = 0; k < 6; ++k) ss >> props[6 * i + k];
  }
  // water IDs after the material blocks (src/read_input.f90:602-611)
  std::vector<char> water(nmat, 0);
  const bool iswater = D.lines.count("water:") != 0;
  if (iswater) {
    int nwmat = 0;
    fm >> nwmat;
    for (int i = 0; i < nwmat; ++i) {
      int id;
      fm >> id;
      water[id - 1] = 1;
    }
  }
  std::vector<int> counts(3, 0), pairs;
  const char* bck[3] = {"uxfile", "uyfile", "uzfile"};
  for (int d = 0; d < 3; ++d) {
    std::ifstream fb(base + D.lines["bc:"][bck[d]]);
    int bctype;
    double val;
    while (fb >> bctype >> val) {
      int nel;
      fb >> nel;
      for (int i = 0; i < nel; ++i) {
        int e, f;
        fb >> e >> f;
        pairs.push_back(e); pairs.push_back(f);
        counts[d]++;
      }
    }
  }
  OrcModel* h = (OrcModel*)orc_model_from_hex8(nnode8, xyz[0].data(), xyz[1].data(), xyz[2].data(), nelmt,
                                                conn.data(), mid.data(), nmat, props.data(), counts.data(),
                                                pairs.data());
  auto& ctl = D.lines["control:"];
  Control& C = h->C;
  C.cg_tol = ZEROTOL; C.cg_maxiter = 100; C.nl_tol = ZEROTOL; C.nl_maxiter = 100;  // src/read_input.f90:109-110
  if (ctl.count("cg_tol")) C.cg_tol = std::atof(ctl["cg_tol"].c_str());
  if (ctl.count("cg_maxiter")) C.cg_maxiter = std::atoi(ctl["cg_maxiter"].c_str());
  if (ctl.count("nl_tol")) C.nl_tol = std::atof(ctl["nl_tol"].c_str());
  if (ctl.count("nl_maxiter")) C.nl_maxiter = std::atoi(ctl["nl_maxiter"].c_str());
  if (ctl.count("phinu")) C.phinu = std::atoi(ctl["phinu"].c_str()) == 1;
  int nsrf = ctl.count("nsrf") ? std::atoi(ctl["nsrf"].c_str()) : 1;
  h->srf_list.assign(nsrf, 1.0);
  if (ctl.count("srf")) {
    std::stringstream ss(ctl["srf"]);
    for (int i = 0; i < nsrf; ++i) ss >> h->srf_list[i];
  }
  if (D.lines["material:"].count("allelastic")) C.allelastic = std::atoi(D.lines["material:"]["allelastic"].c_str()) == 1;
  if (D.lines.count("eqload:")) {  // src/read_input.f90:293-303
    auto& eq = D.lines["eqload:"];
    C.iseqload = 1;
    C.eqkx = eq.count("eqkx") ? std::atof(eq["eqkx"].c_str()) : 0.0;
    C.eqky = eq.count("eqky") ? std::atof(eq["eqky"].c_str()) : 0.0;
    C.eqkz = eq.count("eqkz") ? std::atof(eq["eqkz"].c_str()) : 0.0;
  }
  if (iswater) {  // src/slope.F90:173-187
    std::string tag;
    if (compute_pressure(h->M, water, base + D.lines["water:"]["wsfile"], tag) != 0) {
      delete h;
      return nullptr;
    }
  }
  return h;
}

void orc_free(void* h) { delete (OrcModel*)h; }

// Water table: water_ids (1-based, nwmat) and a water-surface file
// (src/compute_pressure.f90:10-186).  Returns 0, or -1 with errtag (250 chars).
int orc_set_water(void* hv, const int* water_ids, int nwmat, const char* wsfile, char* errtag) {
  OrcModel* h = (OrcModel*)hv;
  std::vector<char> water(h->M.nmatblk, 0);
  for (int i = 0; i < nwmat; ++i) water[water_ids[i] - 1] = 1;
  std::string tag;
  int st = compute_pressure(h->M, water, wsfile, tag);
  if (errtag) std::snprintf(errtag, 250, "%s", tag.c_str());
  return st;
}

// Pore pressure per node and submerged flags (either may be NULL).
// Returns 0 when a water table is set, else -1.
int orc_pore_pressure(void* hv, double* wpressure, int* submerged) {
  OrcModel* h = (OrcModel*)hv;
  if (!h->M.iswater) return -1;
  for (int n = 0; n < h->M.nnode; ++n) {
    if (wpressure) wpressure[n] = h->M.wpressure[n];
    if (submerged) submerged[n] = h->M.submerged[n];
  }
  return 0;
}

// Valency-averaged nodal stress (src/slope.F90:419-437): stress_global(:,num) +=
// stress_elmt(:,:,e) over the elements in order, then divided by node_valency.
void orc_nodal_stress(void* hv, const double* stress_elmt, double* stress_global) {
  const Model& M = ((OrcModel*)hv)->M;
  std::vector<int> valency(M.nnode, 0);
  for (int n = 0; n < M.nnode * NST; ++n) stress_global[n] = 0.0;
  for (int e = 0; e < M.nelmt; ++e)
    for (int a = 0; a < NGLL; ++a) {
      const int n = M.g_num[(size_t)e * NGLL + a];
      valency[n]++;
      for (int c = 0; c < NST; ++c)
        stress_global[(size_t)n * NST + c] = stress_global[(size_t)n * NST + c] + stress_elmt[((size_t)e * NGLL + a) * NST + c];
    }
  for (int n = 0; n < M.nnode; ++n)
    for (int c = 0; c < NST; ++c) stress_global[(size_t)n * NST + c] = stress_global[(size_t)n * NST + c] / (double)valency[n];
}
void orc_set_dot_order(int order) { g_dot_order = order; }

void orc_model_sizes(void* hv, int* out /* nnode nelmt neq nmatblk nsrf */) {
  OrcModel* h = (OrcModel*)hv;
  out[0] = h->M.nnode; out[1] = h->M.nelmt; out[2] = h->M.neq; out[3] = h->M.nmatblk;
  out[4] = (int)h->srf_list.size();
}
void orc_model_arrays(void* hv, double* g_coord, int* g_num, int* gdof, int* gdof_elmt, int* mat_id) {
  OrcModel* h = (OrcModel*)hv;
  const Model& M = h->M;
  if (g_coord) std::memcpy(g_coord, M.g_coord.data(), sizeof(double) * M.g_coord.size());
  if (g_num) std::memcpy(g_num, M.g_num.data(), sizeof(int) * M.g_num.size());
  if (gdof) std::memcpy(gdof, M.gdof.data(), sizeof(int) * M.gdof.size());
  if (gdof_elmt) std::memcpy(gdof_elmt, M.gdof_elmt.data(), sizeof(int) * M.gdof_elmt.size());
  if (mat_id) std::memcpy(mat_id, M.mat_id.data(), sizeof(int) * M.mat_id.size());
}
void orc_model_control(void* hv, double* dctl /* cg_tol nl_tol */, int* ictl /* cg_maxiter nl_maxiter phinu allelastic */,
                       double* srf) {
  OrcModel* h = (OrcModel*)hv;
  dctl[0] = h->C.cg_tol; dctl[1] = h->C.nl_tol;
  ictl[0] = h->C.cg_maxiter; ictl[1] = h->C.nl_maxiter; ictl[2] = h->C.phinu; ictl[3] = h->C.allelastic;
  if (srf) std::memcpy(srf, h->srf_list.data(), sizeof(double) * h->srf_list.size());
}
void orc_set_control(void* hv, double cg_tol, int cg_maxiter, double nl_tol, int nl_maxiter, int phinu,
                     int allelastic) {
  OrcModel* h = (OrcModel*)hv;
  h->C.cg_tol = cg_tol; h->C.cg_maxiter = cg_maxiter; h->C.nl_tol = nl_tol; h->C.nl_maxiter = nl_maxiter;
  h->C.phinu = phinu; h->C.allelastic = allelastic;
}

// Element stiffness, diagonal and gravity load over all elements.
void orc_stiffness_bodyload(void* hv, double* storekm, double* dprecon, double* extload) {
  OrcModel* h = (OrcModel*)hv;
  stiffness_bodyload(h->M, nullptr, h->M.nelmt, h->M.nu.data(), storekm, dprecon, extload, true,
                     h->C.iseqload != 0, h->C.eqkx, h->C.eqky, h->C.eqkz, h->M.gdof_elmt.data());
}

// Pseudo-static earthquake load factors (the eqload: line, src/read_input.f90:293-303).
void orc_set_eqload(void* hv, double eqkx, double eqky, double eqkz) {
  OrcModel* h = (OrcModel*)hv;
  h->C.iseqload = 1;
  h->C.eqkx = eqkx; h->C.eqky = eqky; h->C.eqkz = eqkz;
}

int orc_pcg_solver(int neq, int nelmt, const double* k, double* u, const double* f, const double* dprecon,
                   const int* gdof_elmt, int cg_maxiter, double cg_tol, int* cg_iter) {
  return pcg_solver(neq, nelmt, k, u, f, dprecon, gdof_elmt, cg_maxiter, cg_tol, cg_iter);
}

// pcg_solver in the GPU drop-in's evaluation order (a checker of the device
// kernels' arithmetic, see pcg_solver_gpu_order)
int orc_pcg_solver_gpu_order(int neq, int nelmt, const double* k, double* u, const double* f, const double* dprecon,
                             const int* gdof_elmt, int cg_maxiter, double cg_tol, int* cg_iter) {
  return pcg_solver_gpu_order(neq, nelmt, k, u, f, dprecon, gdof_elmt, cg_maxiter, cg_tol, cg_iter);
}

void orc_ebe_apply(int neq, int nelmt, const double* k, const double* p, const int* gdof_elmt, double* kp) {
  ebe_apply(neq, nelmt, k, p, gdof_elmt, kp);
}

// One stress/yield/flow/body-load pass (the extracted src/slope.F90:311-383 block).
// One pass of the stress block over elist (1-based, nel; NULL: all elements)
// in the slope form (form 0) or the excavation form (form 1: pore pressure
// before the stored stress, vmeps/scf accumulated when finalising).
double orc_stress_update(void* hv, const int* elist, int nel, int form, const double* x, const double* ymf,
                         const double* nuf, const double* phif, const double* cohf, const double* psif, double dt,
                         int nl_isconv, int finalize, double* evpt, double* stress_elmt, double* bodyload,
                         double* vmeps, double* scf) {
  OrcModel* h = (OrcModel*)hv;
  std::vector<int> el0;
  if (elist) {
    el0.resize(nel);
    for (int i = 0; i < nel; ++i) el0[i] = elist[i] - 1;
  } else {
    nel = h->M.nelmt;
  }
  return stress_update(h->M, elist ? el0.data() : nullptr, nel, x, h->M.gdof_elmt.data(), ymf, nuf, phif, cohf,
                       psif, dt, nl_isconv != 0, finalize != 0, evpt, stress_elmt, bodyload,
                       form == 1 ? vmeps : nullptr, form == 1 ? scf : nullptr, form == 1);
}

void orc_elastic_stress(void* hv, const double* x, double* stress_elmt) {
  OrcModel* h = (OrcModel*)hv;
  elastic_stress(h->M, h->M.gdof_elmt.data(), h->M.ym.data(), h->M.nu.data(), x, stress_elmt);
}

void orc_overburden_stress(void* hv, double z0, double p0, double k0, double* stress_elmt) {
  overburden_stress(((OrcModel*)hv)->M, z0, p0, k0, stress_elmt);
}

int orc_strength_reduction(double srf, int phinu, int nmat, const double* coh, const double* nu, const double* phi,
                           const double* psi, double* cohf, double* nuf, double* phif, double* psif) {
  return strength_reduction(srf, phinu != 0, nmat, coh, nu, phi, psi, cohf, nuf, phif, psif);
}
double orc_dt_viscoplas(int nmat, const double* nuf, const double* phif, const double* ymf) {
  return dt_viscoplas(nmat, nuf, phif, ymf, nullptr);
}

// One full SRF trial of slope3d; res = [srf cg_tot nl_iter converged failed uxmax umax fmax uerr errcode].
// x_out (neq+1) optional; nl_cg (nl_maxiter) optional per-NL-iteration cg counts.
void orc_slope_trial(void* hv, double srf, double* res, double* x_out, double* stress_out, int* nl_cg) {
  OrcModel* h = (OrcModel*)hv;
  if (!h->setup_done) { slope_setup(h->M, h->C, h->S); h->setup_done = true; }
  TrialResult R = slope_trial(h->M, h->C, h->S, srf);
  res[0] = R.srf; res[1] = R.cg_tot; res[2] = R.nl_iter; res[3] = R.converged; res[4] = R.failed;
  res[5] = R.uxmax; res[6] = R.umax; res[7] = R.fmax; res[8] = R.uerr; res[9] = R.errcode;
  if (x_out) std::memcpy(x_out, h->S.x.data(), sizeof(double) * h->S.x.size());
  if (stress_out) std::memcpy(stress_out, h->S.stress.data(), sizeof(double) * h->S.stress.size());
  if (nl_cg) for (size_t i = 0; i < h->S.nl_cg_log.size(); ++i) nl_cg[i] = h->S.nl_cg_log[i];
}

// uerr of every plastic iteration of the last trial (the convergence margin of
// src/slope.F90:307-310); returns the number of entries
int orc_last_uerr_log(void* hv, double* out) {
  OrcModel* h = (OrcModel*)hv;
  if (out) std::memcpy(out, h->S.uerr_log.data(), sizeof(double) * h->S.uerr_log.size());
  return (int)h->S.uerr_log.size();
}

// The slope3d SRF sweep: runs srf[0..nsrf) in order and stops after the first
// trial with nl_iter == nl_maxiter (src/slope.F90:244-443).  Returns the number
// of trials run; res is nsrf x 10 as in orc_slope_trial.
int orc_slope_sweep(void* hv, int nsrf, const double* srf, double* res) {
  OrcModel* h = (OrcModel*)hv;
  int n = 0;
  for (int i = 0; i < nsrf; ++i) {
    orc_slope_trial(hv, srf[i], res + 10 * i, nullptr, nullptr, nullptr);
    ++n;
    if (res[10 * i + 9] != 0) break;
    if (res[10 * i + 4] != 0) break;
  }
  (void)h;
  return n;
}

// Critical SRF by bisection over the grid lo + step*m (m = 0..M), assuming the
// trial at lo is stable and the trial at hi fails; the answer is the smallest
// grid SRF whose trial fails.  Returns the critical SRF; ntrials_out counts trials.
double orc_fos_bisection(void* hv, double lo, double hi, double step, int* ntrials_out) {
  int M = (int)std::lround((hi - lo) / step);
  int a = 0, b = M, nt = 0;
  double res[10];
  while (b - a > 1) {
    int m = (a + b) / 2;
    orc_slope_trial(hv, lo + step * m, res, nullptr, nullptr, nullptr);
    ++nt;
    if (res[4] != 0) b = m; else a = m;
  }
  if (ntrials_out) *ntrials_out = nt;
  return lo + step * b;
}

// ---- known-answer helpers for the tests ----
void orc_tables(double* gll_w /*27*/, double* dlag /*3*27*27*/, double* dshape /*3*8*27*/, int* gnode /*8*/,
                int* faces /*6*9*/) {
  const Tables& T = tables();
  std::memcpy(gll_w, T.gll_weights, sizeof(T.gll_weights));
  std::memcpy(dlag, T.dlagrange, sizeof(T.dlagrange));
  std::memcpy(dshape, T.dshape, sizeof(T.dshape));
  for (int a = 0; a < 8; ++a) gnode[a] = T.hex8_gnode[a];
  for (int f = 0; f < 6; ++f) for (int k = 0; k < 9; ++k) faces[9 * f + k] = T.face_nodes[f][k];
}
void orc_cmat(double E, double nu, double* c) { compute_cmat(E, nu, (double(*)[6])c); }
void orc_stress_invariant(const double* s, double* out) { stress_invariant(s, out[0], out[1], out[2]); }

// Principal stresses, maximum shear and normal stress per node
// (src/postprocess.f90:146-183; rquick_sort src/math_library.f90:211-228).
void orc_principal_stress(int nnode, const double* stress_global, double* psigma, double* taumax, double* nsigma) {
  const double pi = 3.141592653589793, two_third = 2.0 / 3.0;
  for (int n = 0; n < nnode; ++n) {
    double sigm, dsbar, theta;
    stress_invariant(stress_global + (size_t)6 * n, sigm, dsbar, theta);
    double x[3];
    x[0] = sigm + two_third * dsbar * std::sin(theta - two_third * pi);
    x[1] = sigm + two_third * dsbar * std::sin(theta);
    x[2] = sigm + two_third * dsbar * std::sin(theta + two_third * pi);
    for (int i = 1; i < 3; ++i) {
      double temp = x[i];
      int j = i - 1;
      while (j >= 0 && x[j] > temp) { x[j + 1] = x[j]; j = j - 1; }
      x[j + 1] = temp;
    }
    for (int c = 0; c < 3; ++c) psigma[3 * n + c] = x[c];
    taumax[n] = 0.5 * std::fabs(x[0] - x[2]);
    nsigma[n] = 0.5 * (x[0] + x[2]);
  }
}
double orc_mohcouf(double phi, double c, double sigm, double dsbar, double theta) {
  return mohcouf(phi, c, sigm, dsbar, theta);
}
void orc_mohcouq(double psi, double dsbar, double theta, double* dq) { mohcouq(psi, dsbar, theta, dq[0], dq[1], dq[2]); }
void orc_formm(const double* s, double* m) {
  formm(s, (double(*)[6])m, (double(*)[6])(m + 36), (double(*)[6])(m + 72));
}

// ---------------------------------------------------------------------------
// excavation3d (src/excavation.F90:15-709), s0_type 0 or 1, nsrf=1.
// res per stage: [stage cg_tot nl_tot uxmax umax fmax failed errcode].
// Returns the number of stages run.
// ---------------------------------------------------------------------------
int orc_excavation(void* hv, int s0_type, double z0, double s0, double k0, int nexcav, const int* nexcavid,
                   const int* excavid, int ninc, double srf, double* res, double* x_last, double* vmeps_out,
                   double* scf_out) {
  OrcModel* h = (OrcModel*)hv;
  {
    // the stage index of src/excavation.F90:339 must stay inside excavid
    long long total = 0;
    for (int is = 0; is < nexcav; ++is) total += nexcavid[is];
    for (int is = 0; is < nexcav; ++is)
      if (nexcavid[is] < 1 || (long long)is * nexcavid[is] + nexcavid[is] > total) return -2;
  }
  Model M = h->M;  // gdof is renumbered per stage
  const Control& C = h->C;
  const int nel = M.nelmt, nm = M.nmatblk;
  std::vector<double> stress((size_t)NST * NGLL * nel, 0.0), evpt((size_t)NST * NGLL * nel, 0.0);
  if (s0_type == 0) {
    const int n1 = M.neq + 1;
    std::vector<double> km((size_t)NEDOF * NEDOF * nel), dp(n1), ext(n1, 0.0), x(n1, 0.0);
    stiffness_bodyload(M, nullptr, nel, M.nu.data(), km.data(), dp.data(), ext.data(), true, false, 0, 0, 0,
                       M.gdof_elmt.data());
    for (int i = 1; i < n1; ++i) dp[i] = ONE / dp[i];
    dp[0] = 0.0;
    int it;
    if (pcg_solver(M.neq, nel, km.data(), x.data(), ext.data(), dp.data(), M.gdof_elmt.data(), C.cg_maxiter,
                   C.cg_tol, &it) != 0)
      return -1;
    x[0] = 0.0;
    elastic_stress(M, M.gdof_elmt.data(), M.ym.data(), M.nu.data(), x.data(), stress.data());
  } else {
    overburden_stress(M, z0, s0, k0, stress.data());
  }
  std::vector<unsigned char> ismat(nm, 1);
  std::vector<double> nodalu((size_t)3 * M.nnode, 0.0);
  int nelmt_intact = nel, nstage = 0;
  for (int is = 0; is < nexcav; ++is) {
    int id0 = is * nexcavid[is], id1 = id0 + nexcavid[is] - 1;  // src/excavation.F90:339 (quirk kept)
    std::vector<unsigned char> off(nm, 0);
    for (int i = id0; i <= id1; ++i) { ismat[excavid[i] - 1] = 0; off[excavid[i] - 1] = 1; }
    std::vector<int> eint, evoid;
    for (int e = 0; e < nel; ++e) {
      int im = M.mat_id[e] - 1;
      if (off[im]) evoid.push_back(e);
      else if (ismat[im]) eint.push_back(e);
    }
    nelmt_intact = (int)eint.size();
    if (nelmt_intact <= 0) break;
    std::vector<char> isnode(M.nnode, 0);
    for (int e : eint) for (int a = 0; a < NGLL; ++a) isnode[M.g_num[(size_t)e * NGLL + a]] = 1;
    // per-stage fields (src/excavation.F90:335): vmeps = 0, scf = inftol
    std::vector<double> vmeps(M.nnode, 0.0), scf(M.nnode, INFTOL);
    // modify_gdof (src/excavation_library.f90:90-111)
    for (int j = 0; j < M.nnode; ++j) if (!isnode[j]) for (int d = 0; d < 3; ++d) M.gdof[(size_t)3 * j + d] = 0;
    int neq = 0;
    for (int j = 0; j < M.nnode; ++j)
      for (int d = 0; d < 3; ++d) if (M.gdof[(size_t)3 * j + d] != 0) M.gdof[(size_t)3 * j + d] = ++neq;
    M.neq = neq;
    build_gdof_elmt(M);
    const int n1 = neq + 1;
    // excavation_load_nodal (src/excavation_library.f90:186-236) then distribute2ghosts (serial_library.f90:110-130)
    const Tables& T = tables();
    std::vector<double> excavload((size_t)3 * M.nnode, 0.0);
    for (int e : evoid) {
      ElemGeom G;
      elem_coord(M, T.hex8_gnode, e, G);
      double bload[NEDOF] = {0}, eld[NEDOF] = {0};
      int idof = 0;
      for (int i = 0; i < NGLL; ++i) {
        double detjac, deriv[3][NENOD], bmat[6][NEDOF];
        point_deriv(G, i, detjac, deriv);
        compute_bmat(deriv, bmat);
        const double* sg = stress.data() + ((size_t)e * NGLL + i) * NST;
        for (int j = 0; j < NEDOF; ++j) {
          double acc = 0.0;
          for (int s = 0; s < 6; ++s) acc = acc + sg[s] * bmat[s][j];
          bload[j] = bload[j] + acc * detjac * T.gll_weights[i];
        }
        idof += 3;
        eld[idof - 1] = eld[idof - 1] + detjac * T.gll_weights[i];
      }
      double gm = M.gam[M.mat_id[e] - 1];
      for (int a = 0; a < NGLL; ++a) {
        int nd = M.g_num[(size_t)e * NGLL + a];
        for (int d = 0; d < 3; ++d) excavload[(size_t)3 * nd + d] += eld[3 * a + d] * gm + bload[3 * a + d];
      }
    }
    std::vector<double> extload(n1, 0.0);
    for (int j = 0; j < M.nnode; ++j)
      for (int d = 0; d < 3; ++d) extload[M.gdof[(size_t)3 * j + d]] = excavload[(size_t)3 * j + d];
    extload[0] = 0.0;
    std::vector<double> cohf(nm), nuf(nm), phif(nm), psif(nm);
    strength_reduction(srf, C.phinu != 0, nm, M.coh.data(), M.nu.data(), M.phi.data(), M.psi.data(), cohf.data(),
                       nuf.data(), phif.data(), psif.data());
    double dt = dt_viscoplas(nm, nuf.data(), phif.data(), M.ym.data(), ismat.data());
    std::vector<double> km((size_t)NEDOF * NEDOF * nelmt_intact), dp(n1);
    stiffness_bodyload(M, eint.data(), nelmt_intact, nuf.data(), km.data(), dp.data(), nullptr, false, false, 0, 0,
                       0, M.gdof_elmt.data());
    dp[0] = 0.0;
    for (int i = 1; i < n1; ++i) dp[i] = ONE / dp[i];
    std::vector<int> ge_int((size_t)NEDOF * nelmt_intact);
    for (int ie = 0; ie < nelmt_intact; ++ie)
      std::memcpy(&ge_int[(size_t)ie * NEDOF], &M.gdof_elmt[(size_t)eint[ie] * NEDOF], sizeof(int) * NEDOF);
    for (int i = 0; i < n1; ++i) extload[i] = extload[i] / ninc;
    int cg_tot = 0, nl_tot = 0, nl_iter = 0;
    double fmax = 0;
    std::vector<double> bodyload(n1), load(n1), x(n1), oldx(n1);
    int errcode = 0;
    for (int inc = 0; inc < ninc; ++inc) {
      std::fill(bodyload.begin(), bodyload.end(), 0.0);
      std::fill(evpt.begin(), evpt.end(), 0.0);
      std::fill(x.begin(), x.end(), 0.0);
      std::fill(oldx.begin(), oldx.end(), 0.0);
      bool nl_isconv = false;
      for (nl_iter = 1; nl_iter <= C.nl_maxiter; ++nl_iter) {
        fmax = 0.0;
        for (int i = 0; i < n1; ++i) load[i] = extload[i] + bodyload[i];
        load[0] = 0.0;
        int cg_iter;
        errcode = pcg_solver(neq, nelmt_intact, km.data(), x.data(), load.data(), dp.data(), ge_int.data(),
                             C.cg_maxiter, C.cg_tol, &cg_iter);
        if (errcode != 0) break;
        cg_tot += cg_iter;
        x[0] = 0.0;
        double num = 0, den = 0;
        for (int i = 0; i < n1; ++i) { num = std::max(num, std::fabs(x[i] - oldx[i])); den = std::max(den, std::fabs(x[i])); }
        double uerr = num / den;
        oldx = x;
        nl_isconv = uerr <= C.nl_tol;
        bool fin = nl_isconv || nl_iter == C.nl_maxiter;
        fmax = stress_update(M, eint.data(), nelmt_intact, x.data(), M.gdof_elmt.data(), M.ym.data(), nuf.data(),
                             phif.data(), cohf.data(), psif.data(), dt, nl_isconv, fin, evpt.data(), stress.data(),
                             bodyload.data(), vmeps.data(), scf.data(), true);
        if (fin) break;
      }
      if (errcode != 0) break;
      nl_tot += nl_iter;
      for (int j = 0; j < M.nnode; ++j)
        for (int d = 0; d < 3; ++d) {
          int g = M.gdof[(size_t)3 * j + d];
          if (g) nodalu[(size_t)3 * j + d] += x[g];
        }
      if (x_last && is == nexcav - 1 && inc == ninc - 1) std::memcpy(x_last, x.data(), sizeof(double) * n1);
    }
    // average effective plastic strain over the intact valency (src/excavation.F90:656-661)
    {
      std::vector<int> valency(M.nnode, 0);
      for (int e : eint) for (int a = 0; a < NGLL; ++a) valency[M.g_num[(size_t)e * NGLL + a]]++;
      for (int j = 0; j < M.nnode; ++j)
        if (isnode[j]) vmeps[j] = vmeps[j] / (double)valency[j];
      if (vmeps_out) std::memcpy(vmeps_out, vmeps.data(), sizeof(double) * M.nnode);
      if (scf_out) std::memcpy(scf_out, scf.data(), sizeof(double) * M.nnode);
    }
    double uxmax = 0, umax = 0;
    for (int j = 0; j < M.nnode; ++j) {
      if (!isnode[j]) continue;
      double* u = &nodalu[(size_t)3 * j];
      for (int d = 0; d < 3; ++d) uxmax = std::max(uxmax, std::fabs(u[d]));
      umax = std::max(umax, std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
    }
    double* r = res + 8 * is;
    r[0] = is + 1; r[1] = cg_tot; r[2] = nl_tot; r[3] = uxmax; r[4] = umax; r[5] = fmax;
    r[6] = (nl_iter == C.nl_maxiter); r[7] = errcode;
    ++nstage;
    if (errcode != 0 || nl_iter == C.nl_maxiter) break;
  }
  return nstage;
}

}  // extern "C"
