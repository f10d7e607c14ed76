// sg_kernels.cuh -- device-side declarations shared by the kernel and driver
// translation units.
#pragma once

#include "sg_internal.h"

namespace sg {

// Per right-hand-side column PCG scalars (device resident).
struct ColState {
  double rz;      // r.z of the current iterate
  double alpha;   // step length of this iteration
  double beta;    // direction update factor for the next iteration
  double tol;     // stop tolerance (step test) or residual reduction (residual test)
  double rr0;     // |r0|^2 at the start (residual test)
  double maxp, maxu, rr;  // last evaluated max|p|, max|u|, |r|^2
  int active;     // column takes part in this solve
  int done;       // stop test met (or failed)
  int iters;      // iteration at which the column stopped
  int failed;     // reached maxiter without meeting the test
};

// Global PCG control word (device resident).
struct PcgGlobal {
  int all_done;
  int it;         // iterations completed
  int maxiter;
  int mode;       // bit 0: 0 = reference step test, 1 = residual reduction test; bit 1: keep direction
  int kcols;      // columns in use (<= KR)
  unsigned cntB, cntC, pad;
  int err;        // set to 1 by a bounded wait of this solve's kernels that ran out
};

// Factored material block for the stress update, per trial.
struct MatF {
  double c11, c12, c44;  // compute_cmat(ym, nuf) entries (src/elastic.f90:13-42)
  double snph, csph;     // sin, cos of phif (mohcouf, src/plastic_library.f90:95-108)
  double cohf;
  double snps;           // sin of psif (mohcouq, src/plastic_library.f90:116-143)
  double pad;
};

// Kernel launch wrappers (sg_kernels.cu)
long long launch_count();        // kernel launches issued so far (host counter)
void add_launches(long long n);  // kernels launched through a replayed CUDA graph
void set_apply_variant(int v);   // 0 register-staged, 1 TMA pipeline, 2 tensor cores for 8/16 FP32 RHS,
                                 // 3 lane per (element, RHS) for 8/16 FP32 RHS, 4 matrix-free FP32,
                                 // 5 (default) 3 with matrix-free FP32 on small meshes
void set_entry_table(const int* d_entry);
// The element applies that wait on mbarriers set *err to 1 when a bounded
// wait runs out (err is the calling solve's own word, never shared between
// contexts).
template <int KR>
void launch_apply_tc(const float* Ks, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                     float* Y, const ColState* cs, const PcgGlobal* G, const int* d_entry, const int* pos,
                     int* err, cudaStream_t s);
// The search direction formed inside the fused FP32 iteration (combine = 2):
// p = beta p_old + D (r - alpha kp) from the previous step's r, kp and the
// inverted diagonal D, so that the vector update needs no kernel of its own.
struct FusedDir {
  const float* r = nullptr;
  const float* kp = nullptr;
  const float* dinv = nullptr;
};
template <int KR>
void launch_apply_lanes(const float* Ks, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                        float* Y, const ColState* cs, const PcgGlobal* G, const int* pos, int* err, cudaStream_t s,
                        FusedDir fz = FusedDir());
// Fused FP32 PCG step for 8 or 16 columns (see k_pcg_gather_update): gather
// of the element products, the previous step's vector update, the new
// direction and the dots of the next step in one kernel.
template <int KR>
void pcg_gather_update(const GatherTopo& T, const float* Y, float* kp, float* p, float* r, float* u,
                       const float* dinv, ColState* cs, PcgGlobal* G, double* part, cudaStream_t s);
// After a fused solve: p -= D r for the columns that took part, so that the
// direction a later keep_dir solve continues is that of the last step taken.
template <int KR>
void fused_dir_restore(int n1, float* p, const float* r, const float* dinv, const ColState* cs, cudaStream_t s);
bool fused_pcg_enabled();   // SG_FUSED=1 selects the two-kernel iteration
bool apply_uses_lanes(int dense, int KR);  // the FP32 apply of this operator is k_apply_lanes
// Matrix-free FP32 apply (sg_apply_mf.cu): rec holds per GLL point J^-1 and the
// C constants times w detJ; pcg_apply takes it with dense = 2.
template <int KR>
void launch_apply_mf(const float* rec, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                     float* Y, const ColState* cs, const PcgGlobal* G, const int* pos, cudaStream_t s);
void launch_mf_record(const double* geo, const int* mat_id, const int* elist, int nel, const double* ym,
                      const double* nu, float* rec, cudaStream_t s);
constexpr int MF_REC = 12;        // floats per GLL point of the matrix-free record
void launch_nodal_average(const int* ptr, const int* slot, int nnode, const double* stress, double* out,
                          cudaStream_t s);  // sg_output.cu
bool fp32_matrix_free(int nelmt);
// Persistent cooperative FP32 PCG chunk for small meshes (sg_pcg_persist.cu);
// false when it cannot run (the caller launches the separate kernels).
template <int KR>
bool launch_pcg_persistent(const float* rec, const int* ge, int nelmt, const int* pos, const GatherTopo& T, int n1,
                           float* u, float* r, float* z, float* p, float* kp, float* Y, const float* dp,
                           ColState* cs, PcgGlobal* G, double* part, int chunk, cudaStream_t s);
bool persist_enabled();                 // SG_PERSIST=0 turns the persistent chunk off
int persist_max_elements();             // meshes below this use it
// a persistent chunk whose grid barrier timed out sets G->err
void set_gather_variant(int v);  // 1 row-cooperative gather for FP32 with 4/8/16 RHS (default), 0 staged
template <typename V, int KR>
// Y receives element slot (e, a)'s three rows (x KR) at the slot's gather
// position pos[e*27+a] (slots of fully fixed nodes, pos < 0, are skipped).
void pcg_apply(int dense, const void* K, const int* ge, int nelmt, const V* p_old, const V* z, int combine,
               V* Y, const ColState* cs, const PcgGlobal* G, const int* d_nbr, const int* pos, int* err,
               cudaStream_t s);
template <typename V, int KR>
void pcg_gather(const GatherTopo& T, const V* Y, V* kp, V* p, const V* z, int mode, ColState* cs,
                PcgGlobal* G, double* part, cudaStream_t s);
template <typename V, int KR>
void pcg_update(int n1, V* u, V* r, V* z, const V* p, const V* kp, const V* f, const V* dprecon, int init,
                ColState* cs, PcgGlobal* G, double* part, cudaStream_t s);

// Yb layout [nel][81][ystride] at column ycol (ystride = KR of the trial batch)
void launch_stress_update(const double* geo, const int* elist, int nel, const int* ge_glob, const int* mat_id,
                          const double* x, int xstride, int xcol, const MatF* mf, double dt, int nl_isconv,
                          int finalize, double* evpt, double* stress, double* Yb, int ystride, int ycol,
                          double* fmax_part, const int* pos, cudaStream_t s, double* vm_pt = nullptr,
                          double* sf_pt = nullptr, const double* wp = nullptr, const int* gnum = nullptr,
                          int wp_first = 0);
// submerged-node flags and hydrostatic pore pressure per node; err (set to
// INT_MAX by the caller) gets the smallest node + 1 whose free surface cannot
// be determined
void launch_water_pressure(int nnode, int nelmt, const double* g_coord, const int* g_num, const int* mat_id,
                           const int* water_mat, const WaterSurface* surf, int nsurf, const int* face, int* sub,
                           double* wp, int* err, int* nvert, cudaStream_t s);
void launch_elastic_stress(const double* geo, const int* elist, int nel, const int* ge_glob, const int* mat_id,
                           const double* x, int xstride, int xcol, const MatF* mf, int accumulate, double* stress,
                           cudaStream_t s);
void launch_overburden(const double* g_coord, const int* g_num, const int* mat_id, const double* gam, int nelmt,
                       double z0, double p0, double k0, double* stress, cudaStream_t s);
void launch_release_load(const double* geo, const int* elist, int nel, const int* mat_id, const double* gam,
                         const double* stress, double* Ye, const int* pos, cudaStream_t s);
void launch_nl_check(int n1, int KR, int k, const double* x, double* oldx, double* part, cudaStream_t s);
void launch_load_combine(int n1, int KR, const double* extload, const double* bodyload, double* load,
                         cudaStream_t s);
template <typename V>
void launch_gather_plain(const GatherTopo& T, int KR, const V* Y, V* out, int accumulate, const int* colmask,
                         cudaStream_t s);
void launch_final_reduce(const double* part, int nblk, int KR, int nq, int maxmask, double* out, cudaStream_t s);
void launch_disp_max(int nnode, const int* gdof, const double* x, int KR, int col, double* part, cudaStream_t s);
void launch_div(size_t n, double* y, double a, cudaStream_t s);
void launch_col_zero(int n1, int KR, int j, double* a, double* b, double* c, cudaStream_t s);
void launch_residual_norms(int n1, int KR, const double* f, const double* kp, double* r64, float* r32,
                           double* part, cudaStream_t s);
void launch_axpy_correction(int n1, int KR, const int* colmask, const float* d, double* x, double* part,
                            cudaStream_t s);
void launch_invert_diag(int n1, double* dprecon, float* dprecon32, cudaStream_t s);

}  // namespace sg
