// sg_output.cu -- result outputs of the slope and excavation drivers.
//
// * Valency-averaged nodal stress (src/slope.F90:419-437): every node's
//   stress is the sum of the element stresses at that node, taken in element
//   order, divided by the node's valency.  On the device, one thread per node
//   over a node -> element-slot list.
// * Summary file (src/semgeotech.F90:315-319, src/slope.F90:213-220,409-416):
//   banner, control values, and one line per SRF trial
//   "SRF, CGITER, NLITER, UXMAX, UMAX, fmax".  The reference writes these
//   with Fortran list-directed output; the same lines and fields are written
//   here as blank-separated values with full precision.
// * Principal stresses, maximum shear stress and the normal stress on its
//   plane per node (src/postprocess.f90:146-183).
// * EnSight Gold C-binary files (src/visual.f90:75-290,
//   src/semgeotech.F90:126-312, src/postprocess.f90:128-248): the .case
//   file, the geometry with every 27-node element written as its 8 hexa8
//   sub-cells in Exodus corner order, and per-node variables (displacement
//   vector, symmetric stress tensor, scalars), 80-byte text records, 4-byte
//   integers and 4-byte reals, coordinates and components stored one
//   component after the other.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sg_kernels.cuh"

namespace sg {

__global__ void k_nodal_average(const int* __restrict__ ptr, const int* __restrict__ slot, int nnode,
                                const double* __restrict__ stress, double* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnode) return;
  const int a = ptr[n], b = ptr[n + 1];
  double s[NST] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = a; k < b; ++k) {
    const double* st = stress + (size_t)slot[k] * NST;
#pragma unroll
    for (int c = 0; c < NST; ++c) s[c] = s[c] + st[c];
  }
  const double v = (double)(b - a);
#pragma unroll
  for (int c = 0; c < NST; ++c) out[(size_t)n * NST + c] = (b > a) ? s[c] / v : 0.0;
}

void launch_nodal_average(const int* ptr, const int* slot, int nnode, const double* stress, double* out,
                          cudaStream_t s) {
  if (nnode > 0) k_nodal_average<<<(nnode + 255) / 256, 256, 0, s>>>(ptr, slot, nnode, stress, out);
}

}  // namespace sg

namespace {

// one 80-character text record (blank padded, as Fortran's character(len=80))
void rec80(FILE* f, const char* s) {
  char b[80];
  std::memset(b, ' ', sizeof(b));
  std::memcpy(b, s, std::min<size_t>(std::strlen(s), sizeof(b)));
  std::fwrite(b, 1, sizeof(b), f);
}
void i32(FILE* f, int v) { std::fwrite(&v, 4, 1, f); }

// Fortran e12.5 edit descriptor: 0.ddddd mantissa, signed 2-digit exponent
std::string fortran_e12_5(double v) {
  char m[32];
  std::snprintf(m, sizeof(m), "%.4E", v);  // d.ddddE+xx
  const char* p = m;
  const bool neg = (*p == '-');
  if (neg) ++p;
  if (v == 0.0) return "  0.00000E+00";
  const int ex = std::atoi(std::strchr(p, 'E') + 1) + 1;
  char out[32];
  std::snprintf(out, sizeof(out), "%s0.%c%c%c%c%cE%c%02d", neg ? "-" : "", p[0], p[2], p[3], p[4], p[5],
                ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
  char pad[32];
  std::snprintf(pad, sizeof(pad), "%12s", out);
  return pad;
}

// stress invariants of a 6-component stress (src/math_library.f90:144-186):
// mean stress, sqrt(3 J2) with J2 clamped at 1e-12, Lode angle
void invariants(const double* st, double& sigm, double& dsbar, double& theta) {
  const double sq3 = std::sqrt(3.0), small = 1e-12;
  const double s1 = st[0], s2 = st[1], s3 = st[2], s4 = st[3], s5 = st[4], s6 = st[5];
  sigm = (s1 + s2 + s3) / 3.0;
  double d2 = ((s1 - s2) * (s1 - s2) + (s2 - s3) * (s2 - s3) + (s3 - s1) * (s3 - s1)) / 6.0 + s4 * s4 + s5 * s5 +
              s6 * s6;
  if (d2 < small) d2 = small;
  const double ds1 = s1 - sigm, ds2 = s2 - sigm, ds3 = s3 - sigm;
  const double d3 = ds1 * ds2 * ds3 - ds1 * s5 * s5 - ds2 * s6 * s6 - ds3 * s4 * s4 + 2.0 * s4 * s5 * s6;
  dsbar = sq3 * std::sqrt(d2);
  if (dsbar < small) {
    theta = 0.0;
  } else {
    const double r = std::sqrt(d2);
    double sine = -3.0 * sq3 * d3 / (2.0 * (r * r * r));
    if (sine >= 1.0) sine = 1.0;
    if (sine < -1.0) sine = -1.0;
    theta = std::asin(sine) / 3.0;
  }
}

}  // namespace

extern "C" {

int sg_principal_stress(int nnode, const double* stress_global, double* psigma, double* taumax, double* nsigma) {
  if (nnode < 0 || !stress_global || !psigma) return SG_ERR_BADARG;
  const double pi = 3.141592653589793, two_third = 2.0 / 3.0;
  for (int n = 0; n < nnode; ++n) {
    double sigm, dsbar, theta;
    invariants(stress_global + (size_t)6 * n, sigm, dsbar, theta);
    double p[3] = {sigm + two_third * dsbar * std::sin(theta - two_third * pi), sigm + two_third * dsbar * std::sin(theta),
                   sigm + two_third * dsbar * std::sin(theta + two_third * pi)};
    // ascending (compression negative first), insertion sort as rquick_sort
    for (int i = 1; i < 3; ++i) {
      const double t = p[i];
      int j = i - 1;
      while (j >= 0 && p[j] > t) { p[j + 1] = p[j]; --j; }
      p[j + 1] = t;
    }
    for (int c = 0; c < 3; ++c) psigma[(size_t)3 * n + c] = p[c];
    if (taumax) taumax[n] = 0.5 * std::fabs(p[0] - p[2]);
    if (nsigma) nsigma[n] = 0.5 * (p[0] + p[2]);
  }
  return SG_OK;
}

int sg_write_summary_header(const char* path, const sg_control* ctl, int nsrf) {
  if (!path || !ctl || nsrf < 0) return SG_ERR_BADARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return SG_ERR_BADARG;
  std::fprintf(f, " --------------------------------------------\n");
  std::fprintf(f, " Result summary produced by SPECFEM3D_GEOTECH\n");
  std::fprintf(f, " --------------------------------------------\n");
  std::fprintf(f, " CG_MAXITER, CG_TOL, NL_MAXITER, NL_TOL\n");
  std::fprintf(f, " %d %.17g %d %.17g\n", ctl->cg_maxiter, ctl->cg_tol, ctl->nl_maxiter, ctl->nl_tol);
  std::fprintf(f, " Number of SRFs\n");
  std::fprintf(f, " %d\n", nsrf);
  std::fprintf(f, " SRF, CGITER, NLITER, UXMAX, UMAX, fmax\n");
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BADARG;
}

int sg_write_summary_row(const char* path, const sg_trial_result* r) {
  if (!path || !r) return SG_ERR_BADARG;
  FILE* f = std::fopen(path, "a");
  if (!f) return SG_ERR_BADARG;
  std::fprintf(f, " %.17g %d %d %.17g %.17g %.17g\n", r->srf, r->cg_tot, r->nl_iter, r->uxmax, r->umax, r->fmax);
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BADARG;
}

int sg_write_ensight_case(const char* path, const char* head, int nsteps, const double* times, int tstart) {
  if (!path || !head || nsteps < 1 || !times) return SG_ERR_BADARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return SG_ERR_BADARG;
  const int tw = (int)std::ceil(std::log10((double)nsteps + 1.0));
  const std::string wild(tw, '*');
  std::fprintf(f, "FORMAT\ntype:  ensight gold\n\n");
  std::fprintf(f, "GEOMETRY\nmodel:    %s.geo\n\n", head);
  std::fprintf(f, "VARIABLE\n");
  std::fprintf(f, "vector per node: %10d displacement %s_step%s.dis\n\n", 1, head, wild.c_str());
  std::fprintf(f, "tensor symm per node: %10d stress %s_step%s.sig\n\n", 1, head, wild.c_str());
  std::fprintf(f, "TIME\ntime set:%10d\nnumber of steps:%10d\nfilename start number:%10d\n", 1, nsteps, tstart);
  std::fprintf(f, "filename increment:%10d\ntime values: ", 1);
  for (int i = 0; i < nsteps; ++i) std::fprintf(f, "%s\n", fortran_e12_5(times[i]).c_str());
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BADARG;
}

int sg_write_ensight_geo(const char* path, int nnode, const double* g_coord, int nelmt, const int* g_num) {
  if (!path || nnode < 1 || nelmt < 1 || !g_coord || !g_num) return SG_ERR_BADARG;
  for (size_t i = 0; i < (size_t)nelmt * sg::NGLL; ++i)
    if (g_num[i] < 0 || g_num[i] >= nnode) return SG_ERR_BADARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return SG_ERR_BADARG;
  rec80(f, "C Binary");
  rec80(f, "Created by write_ensight Routine");
  rec80(f, "semfem3d");
  rec80(f, "node id off");
  rec80(f, "element id off");
  rec80(f, "part");
  i32(f, 1);
  rec80(f, "unstructured meshes");
  rec80(f, "coordinates");
  i32(f, nnode);
  std::vector<float> c((size_t)nnode);
  for (int d = 0; d < 3; ++d) {
    for (int n = 0; n < nnode; ++n) c[n] = (float)g_coord[(size_t)3 * n + d];
    std::fwrite(c.data(), 4, c.size(), f);
  }
  rec80(f, "hexa8");
  i32(f, nelmt * 8);
  // sub-cell corners in sequential order, then the Exodus corner order
  // (1,2,4,3,5,6,8,7) of the reference's map2exodus, 1-based node ids
  static const int ex[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  for (int e = 0; e < nelmt; ++e)
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          int seq[8];
          seq[0] = k * 9 + j * 3 + i;
          seq[1] = seq[0] + 1;
          seq[2] = seq[0] + 3;
          seq[3] = seq[2] + 1;
          seq[4] = seq[0] + 9;
          seq[5] = seq[4] + 1;
          seq[6] = seq[4] + 3;
          seq[7] = seq[6] + 1;
          int cell[8];
          for (int q = 0; q < 8; ++q) cell[q] = g_num[(size_t)e * sg::NGLL + seq[ex[q]]] + 1;
          std::fwrite(cell, 4, 8, f);
        }
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BADARG;
}

int sg_write_ensight_var(const char* path, const char* description, int ncomp, int nnode, const double* var) {
  if (!path || !description || !var || nnode < 1 || (ncomp != 1 && ncomp != 3 && ncomp != 6)) return SG_ERR_BADARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return SG_ERR_BADARG;
  rec80(f, description);
  rec80(f, "part");
  i32(f, 1);
  rec80(f, "coordinates");
  std::vector<float> c((size_t)nnode);
  for (int d = 0; d < ncomp; ++d) {
    for (int n = 0; n < nnode; ++n) c[n] = (float)var[(size_t)ncomp * n + d];
    std::fwrite(c.data(), 4, c.size(), f);
  }
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BADARG;
}

}  // extern "C"
