// sg_kernels.cu -- sm_103a kernels of the solve path.
//
//   apply     element-by-element operator Y_e = K_e p_e (src/solver.f90:53-58):
//             dense FP64 81x81 (the drop-in's caller-provided matrices) and the
//             sparse symmetric GLL layout (FP64 or FP32, 1..16 right-hand sides)
//   gather    deterministic scatter-add: every free dof sums its element
//             contributions in increasing element order, fused with the PCG
//             direction update and the p.kp dot (src/solver.f90:53-62)
//   update    fused u, r, z update, max-norms, r.z and the step stop test
//             (src/solver.f90:63-73) with last-block finalisation
//   geometry  Jacobian inverse and determinant per GLL point (src/preprocess.f90:112-118)
//   stiffness K6, element matrices, diagonal and gravity load (src/preprocess.f90:74-148)
//   stress    K5, strain, Mohr-Coulomb yield, viscoplastic flow and body load
//             (src/slope.F90:311-383, src/excavation.F90:546-616)
//
// All reductions use a fixed grid (NPART blocks) and fixed-order trees, so a
// run is bitwise reproducible on the same device type.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <type_traits>

#include "sg_kernels.cuh"

#include <atomic>

namespace sg {

// host-side count of kernel launches issued by this library
std::atomic<long long> g_launch_count{0};
long long launch_count() { return g_launch_count.load(); }
void add_launches(long long n) { g_launch_count += n; }
#define SG_LAUNCH ++g_launch_count,

// D[p][m] = derivative of the m-th 1D Lagrange polynomial on the GLL points
// {-1, 0, 1} evaluated at point p (lagrange1dGLL, src/gll_library.f90:257-299);
// all entries are exact in binary floating point.
__constant__ double c_D[3][3];
__constant__ double c_w[NGLL];             // gll_weights (src/gll_library.f90:46-60)
__constant__ double c_dshape[3][8][NGLL];  // dshape_hex8 (src/shape_library.f90:104-216)
__constant__ int c_gnode[8];               // hex8_gnode (src/element.f90:21-45)

void upload_constants() {
  static bool done = false;
  if (done) return;
  const double D[3][3] = {{-1.5, 2.0, -0.5}, {-0.5, 0.0, 0.5}, {0.5, -2.0, 1.5}};
  const double xi[3] = {-1.0, 0.0, 1.0}, w1[3] = {1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0};
  double w[NGLL], ds[3][8][NGLL];
  const double e8 = 0.125;
  int n = 0;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i, ++n) {
        w[n] = w1[i] * w1[j] * w1[k];
        double xp = 1 + xi[i], xm = 1 - xi[i], ep = 1 + xi[j], em = 1 - xi[j], zp = 1 + xi[k], zm = 1 - xi[k];
        ds[0][0][n] = -e8 * em * zm; ds[0][1][n] = e8 * em * zm; ds[0][2][n] = e8 * ep * zm; ds[0][3][n] = -e8 * ep * zm;
        ds[0][4][n] = -e8 * em * zp; ds[0][5][n] = e8 * em * zp; ds[0][6][n] = e8 * ep * zp; ds[0][7][n] = -e8 * ep * zp;
        ds[1][0][n] = -e8 * xm * zm; ds[1][1][n] = -e8 * xp * zm; ds[1][2][n] = e8 * xp * zm; ds[1][3][n] = e8 * xm * zm;
        ds[1][4][n] = -e8 * xm * zp; ds[1][5][n] = -e8 * xp * zp; ds[1][6][n] = e8 * xp * zp; ds[1][7][n] = e8 * xm * zp;
        ds[2][0][n] = -e8 * xm * em; ds[2][1][n] = -e8 * xp * em; ds[2][2][n] = -e8 * xp * ep; ds[2][3][n] = -e8 * xm * ep;
        ds[2][4][n] = e8 * xm * em; ds[2][5][n] = e8 * xp * em; ds[2][6][n] = e8 * xp * ep; ds[2][7][n] = e8 * xm * ep;
      }
  const int gn[8] = {0, 2, 8, 6, 18, 20, 26, 24};
  cudaMemcpyToSymbol(c_D, D, sizeof(D));
  cudaMemcpyToSymbol(c_w, w, sizeof(w));
  cudaMemcpyToSymbol(c_dshape, ds, sizeof(ds));
  cudaMemcpyToSymbol(c_gnode, gn, sizeof(gn));
  done = true;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
constexpr unsigned FULL = 0xffffffffu;

template <typename V>
__device__ __forceinline__ V fmav(V a, V b, V c);
template <>
__device__ __forceinline__ double fmav<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmav<float>(float a, float b, float c) { return fmaf(a, b, c); }

// p_new = z + beta*p, rounded the same way wherever it is formed (the apply
// forms it on the fly, the gather stores it).  The FP32 solve stays in FP32
// arithmetic: GB300's FP64 rate is 1/64 of its FP32 rate.
template <typename V>
__device__ __forceinline__ V pdir(V beta, V p, V z) { return fmav<V>(beta, p, z); }

// Dot-product accumulator.  FP64 vectors accumulate in FP64.  FP32 vectors
// accumulate exact products (a*b = p + e with e = fma(a,b,-p)) in a
// compensated two-float sum, which keeps FP64-level accuracy of the sum while
// issuing only FP32 instructions; the pair is widened to FP64 per thread.
template <typename V>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    float t = hi + p;
    float bp = t - hi;
    float err = (hi - (t - bp)) + (p - bp);
    hi = t;
    lo += err + e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Per-column block reduction of `val` (threads whose index = j mod KR hold
// column j).  Result for column j lands in out[j] on thread 0..KR-1 of warp 0.
// op 0 = sum, 1 = max.  Fixed tree order.
template <int KR>
__device__ __forceinline__ double warp_col_reduce(double v, int op) {
#pragma unroll
  for (int o = 16; o >= KR; o >>= 1) {
    double w = __shfl_xor_sync(FULL, v, o);
    v = op ? fmax(v, w) : v + w;
  }
  return v;
}


// Load KR consecutive values (16-byte vector loads when the row allows it).
template <typename V, int KR>
__device__ __forceinline__ void loadv(const V* __restrict__ src, V (&out)[KR]) {
  if constexpr (std::is_same<V, float>::value && KR % 4 == 0) {
#pragma unroll
    for (int q = 0; q < KR / 4; ++q) {
      float4 t = reinterpret_cast<const float4*>(src)[q];
      out[4 * q] = t.x; out[4 * q + 1] = t.y; out[4 * q + 2] = t.z; out[4 * q + 3] = t.w;
    }
  } else if constexpr (std::is_same<V, double>::value && KR % 2 == 0) {
#pragma unroll
    for (int q = 0; q < KR / 2; ++q) {
      double2 t = reinterpret_cast<const double2*>(src)[q];
      out[2 * q] = t.x; out[2 * q + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < KR; ++j) out[j] = src[j];
  }
}



// Store KR consecutive values (16-byte vector stores when the row allows it).
template <typename V, int KR>
__device__ __forceinline__ void storev(V* __restrict__ dst, const V (&v)[KR]) {
  if constexpr (std::is_same<V, float>::value && KR % 4 == 0) {
#pragma unroll
    for (int q = 0; q < KR / 4; ++q)
      reinterpret_cast<float4*>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else if constexpr (std::is_same<V, double>::value && KR % 2 == 0) {
#pragma unroll
    for (int q = 0; q < KR / 2; ++q) reinterpret_cast<double2*>(dst)[q] = make_double2(v[2 * q], v[2 * q + 1]);
  } else {
#pragma unroll
    for (int j = 0; j < KR; ++j) dst[j] = v[j];
  }
}

// Store a node's 3 x KR results (one contiguous run) with 16-byte stores.
template <typename V, int KR>
__device__ __forceinline__ void storev3(V* __restrict__ dst, const V (&acc)[3][KR]) {
  if constexpr (std::is_same<V, float>::value && KR % 4 == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int q = 0; q < KR / 4; ++q)
        reinterpret_cast<float4*>(dst + c * KR)[q] =
            make_float4(acc[c][4 * q], acc[c][4 * q + 1], acc[c][4 * q + 2], acc[c][4 * q + 3]);
  } else if constexpr (std::is_same<V, double>::value && KR % 2 == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int q = 0; q < KR / 2; ++q)
        reinterpret_cast<double2*>(dst + c * KR)[q] = make_double2(acc[c][2 * q], acc[c][2 * q + 1]);
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int j = 0; j < KR; ++j) dst[c * KR + j] = acc[c][j];
  }
}

// last-block election: returns true in the block that finished last.
__device__ __forceinline__ bool last_block(unsigned* counter) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// ---------------------------------------------------------------------------
// Geometry cache: Jacobian of the hex8 map at each GLL point, its determinant
// and its inverse (determinant/invert, src/math_library.f90:66-138).
// geo[(e*27+i)*10 + 3*d + a] = Jinv(d,a); geo[..+9] = detJ.
// ---------------------------------------------------------------------------
__global__ void k_geometry(const double* __restrict__ g_coord, const int* __restrict__ g_num, int nelmt,
                           double* __restrict__ geo) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelmt * NGLL) return;
  int e = t / NGLL, i = t - e * NGLL;
  double coord[8][3];
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    int nd = g_num[(size_t)e * NGLL + c_gnode[g]];
#pragma unroll
    for (int b = 0; b < 3; ++b) coord[g][b] = g_coord[(size_t)3 * nd + b];
  }
  double x[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double s = 0.0;
#pragma unroll
      for (int g = 0; g < 8; ++g) s = __dadd_rn(s, __dmul_rn(c_dshape[a][g][i], coord[g][b]));
      x[a][b] = s;
    }
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
  double* o = geo + (size_t)t * GEO_STRIDE;
  o[0] = j11 / det; o[1] = j12 / det; o[2] = j13 / det;
  o[3] = j21 / det; o[4] = j22 / det; o[5] = j23 / det;
  o[6] = j31 / det; o[7] = j32 / det; o[8] = j33 / det;
  o[9] = det;
}

void launch_geometry(const double* g_coord, const int* g_num, int nelmt, double* geo, cudaStream_t s) {
  int n = nelmt * NGLL;
  SG_LAUNCH k_geometry<<<(n + 127) / 128, 128, 0, s>>>(g_coord, g_num, nelmt, geo);
}

// deriv(:,n) at GLL point i: sum_a Jinv(:,a) dlagrange(a,i,n).  dlagrange is
// non-zero only for nodes on the three lattice lines through i, where it is
// D[i_a][n_a]; the zero terms of the reference sum are skipped (they add +0).
__device__ __forceinline__ bool on_line(int i, int n) {
  int dx = (i % 3) != (n % 3), dy = ((i / 3) % 3) != ((n / 3) % 3), dz = (i / 9) != (n / 9);
  return dx + dy + dz <= 1;
}
__device__ __forceinline__ void point_grad(const double* __restrict__ Ji, int i, int n, double g[3]) {
  int ic[3] = {i % 3, (i / 3) % 3, i / 9}, nc[3] = {n % 3, (n / 3) % 3, n / 9};
  double dl[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    bool same_other = true;
#pragma unroll
    for (int b = 0; b < 3; ++b)
      if (b != a && ic[b] != nc[b]) same_other = false;
    dl[a] = same_other ? c_D[ic[a]][nc[a]] : 0.0;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) s = s + Ji[3 * d + a] * dl[a];
    g[d] = s;
  }
}

// ---------------------------------------------------------------------------
// K6: element stiffness in the sparse symmetric layout.
// K(3n+c,3m+d) = sum_i w_i detJ_i [B_i^T C B_i](3n+c,3m+d) with the isotropic
// C of compute_cmat: for c = d, C11 g_n[c] g_m[c] + C44 sum_{e!=c} g_n[e] g_m[e];
// for c != d, C12 g_n[c] g_m[d] + C44 g_n[d] g_m[c]  (g = deriv columns).
// One block per element; threads loop over the 2430 stored entries.
// ---------------------------------------------------------------------------
constexpr int STIFF_THREADS = 256;

__global__ void __launch_bounds__(STIFF_THREADS) k_stiffness(
    const double* __restrict__ geo, const int* __restrict__ mat_id, const int* __restrict__ elist, int nel,
    const double* __restrict__ ym, const double* __restrict__ nu, const double* __restrict__ gam,
    double* __restrict__ Ks64, float* __restrict__ Ks32, double* __restrict__ Ydiag, double* __restrict__ Ygrav,
    const int* __restrict__ entry, const int* __restrict__ pos, int pseudoeq, double eqkx, double eqky,
    double eqkz) {
  __shared__ double sg[NGLL][NGLL][3];   // grad of node n at point i (zero off the lines)
  __shared__ double sgeo[NGLL][GEO_STRIDE];
  __shared__ double swd[NGLL];
  const int le = blockIdx.x;
  if (le >= nel) return;
  const int e = elist ? elist[le] : le;
  const int im = mat_id[e] - 1;
  // compute_cmat (src/elastic.f90:13-42)
  const double E = ym[im], v = nu[im];
  const double onepv = 1.0 + v, onemv = 1.0 - v, onem2v = 1.0 - 2.0 * v;
  const double Ef = E / (onepv * onem2v);
  const double c11 = onemv * Ef, c12 = v * Ef, c44 = 0.5 * onem2v * Ef;
  for (int t = threadIdx.x; t < NGLL * GEO_STRIDE; t += blockDim.x)
    sgeo[t / GEO_STRIDE][t % GEO_STRIDE] = geo[(size_t)e * NGLL * GEO_STRIDE + t];
  __syncthreads();
  for (int t = threadIdx.x; t < NGLL; t += blockDim.x) swd[t] = sgeo[t][9] * c_w[t];
  for (int t = threadIdx.x; t < NGLL * NGLL; t += blockDim.x) {
    int i = t / NGLL, n = t % NGLL;
    double g[3] = {0.0, 0.0, 0.0};
    if (on_line(i, n)) point_grad(sgeo[i], i, n, g);
    sg[i][n][0] = g[0]; sg[i][n][1] = g[1]; sg[i][n][2] = g[2];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < KS_NNZ; t += blockDim.x) {
    int pk = entry[t];
    int row = pk & 255, col = pk >> 8;
    int n = row / 3, c = row % 3, m = col / 3, d = col % 3;
    if (n == m && c > d) { int tmp = c; c = d; d = tmp; }  // exact symmetry inside own-node blocks
    double acc = 0.0;
    for (int i = 0; i < NGLL; ++i) {
      if (!on_line(i, n) || !on_line(i, m)) continue;
      const double* gn = sg[i][n];
      const double* gm = sg[i][m];
      double b;
      if (c == d) {
        int e1 = (c + 1) % 3, e2 = (c + 2) % 3;
        b = c11 * gn[c] * gm[c] + c44 * (gn[e1] * gm[e1] + gn[e2] * gm[e2]);
      } else {
        b = c12 * gn[c] * gm[d] + c44 * gn[d] * gm[c];
      }
      acc = acc + b * swd[i];
    }
    size_t o = (size_t)le * KS_STRIDE + t;
    if (Ks64) Ks64[o] = acc;
    if (Ks32) Ks32[o] = (float)acc;
    if (row == col && Ydiag) {
      int ps = pos[(size_t)le * NGLL + row / 3];
      if (ps >= 0) Ydiag[(size_t)ps * 3 + row % 3] = acc;
    }
  }
  if (Ks64 || Ks32)
    for (int t = KS_NNZ + threadIdx.x; t < KS_STRIDE; t += blockDim.x) {
      if (Ks64) Ks64[(size_t)le * KS_STRIDE + t] = 0.0;
      if (Ks32) Ks32[(size_t)le * KS_STRIDE + t] = 0.0f;
    }
  // gravity: extload(egdof) -= eld*gam, eld non-zero on z dofs = detJ*w
  // (src/preprocess.f90:123-136); stored as the negated contribution.
  if (Ygrav)
    for (int t = threadIdx.x; t < NEDOF; t += blockDim.x) {
      int a = t / 3, d = t % 3;
      int ps = pos[(size_t)le * NGLL + a];
      if (ps < 0) continue;
      double v = (d == 2) ? -(swd[a] * gam[im]) : -0.0;
      // pseudo-static earthquake load (src/preprocess.f90:137-143):
      // eqload = eqk * eld (eld = w detJ at the node's z entry), times gamma
      if (pseudoeq) v = v + ((d == 0 ? eqkx : d == 1 ? eqky : eqkz) * swd[a]) * gam[im];
      Ygrav[(size_t)ps * 3 + d] = v;
    }
}

void launch_stiffness(const double* geo, const int* mat_id, const int* elist, int nel, const double* ym,
                      const double* nu, const double* gam, double* Ks64, float* Ks32, double* Ydiag,
                      double* Ygrav, const int* d_entry, const int* pos, cudaStream_t s, int pseudoeq,
                      double eqkx, double eqky, double eqkz) {
  if (nel <= 0) return;
  SG_LAUNCH k_stiffness<<<nel, STIFF_THREADS, 0, s>>>(geo, mat_id, elist, nel, ym, nu, gam, Ks64, Ks32, Ydiag, Ygrav,
                                           d_entry, pos, pseudoeq, eqkx, eqky, eqkz);
}

// Expand the sparse symmetric layout to the reference's dense column-major
// 81x81 storage (for export and for checks).
__global__ void k_expand_dense(const double* __restrict__ Ks, int nel, double* __restrict__ dense,
                               const int* __restrict__ entry) {
  int e = blockIdx.x;
  if (e >= nel) return;
  double* D = dense + (size_t)e * NEDOF * NEDOF;
  for (int t = threadIdx.x; t < NEDOF * NEDOF; t += blockDim.x) D[t] = 0.0;
  __syncthreads();
  for (int t = threadIdx.x; t < KS_NNZ; t += blockDim.x) {
    int pk = entry[t], row = pk & 255, col = pk >> 8;
    double v = Ks[(size_t)e * KS_STRIDE + t];
    D[(size_t)col * NEDOF + row] = v;
    D[(size_t)row * NEDOF + col] = v;
  }
}

void launch_expand_dense(const double* Ks64, int nel, double* dense, const int* d_entry, cudaStream_t s) {
  if (nel > 0) SG_LAUNCH k_expand_dense<<<nel, 256, 0, s>>>(Ks64, nel, dense, d_entry);
}

// ---------------------------------------------------------------------------
// Element apply.
// ---------------------------------------------------------------------------
constexpr int APPLY_WARPS = 4;
// 0 = register-staged loads, 1 = TMA bulk-copy pipeline (node lanes),
// 2 = tensor cores (FP32, 8/16 RHS), 3 = lane per (element, RHS) for FP32
// with 8/16 RHS and the TMA node-lane pipeline otherwise (default),
// 4 = as 3 for FP64, matrix-free for the FP32 operator of the mixed solve,
// 5 = as 3, except that the FP32 operator of meshes below MF_AUTO_MAX elements
// is matrix-free (default): on small meshes the PCG iteration is latency-
// bound and the matrix-free apply has the shorter dependency chain (33.6
// against 50.2 us per iteration at 270 elements, 125 against 162 us at 10k);
// at 192k elements the two applies take the same time.
constexpr int MF_AUTO_MAX = 100000;
int g_apply_variant = 5;
void set_apply_variant(int v) { g_apply_variant = v; }
bool fp32_matrix_free(int nelmt) { return g_apply_variant == 4 || (g_apply_variant == 5 && nelmt < MF_AUTO_MAX); }
// device copy of the stored-entry table, needed by the tensor-core apply
const int* g_entry_dev = nullptr;
void set_entry_table(const int* d_entry) { g_entry_dev = d_entry; }

// Dense FP64 81x81, one right-hand side (the drop-in).  One warp per element,
// lane l owns rows l, l+32, l+64; column c of K_e is 81 contiguous doubles,
// read once with a streaming hint.  combine: p_e = z_e + beta*p_old_e.
__global__ void __launch_bounds__(APPLY_WARPS * 32) k_apply_dense64(
    const double* __restrict__ K, const int* __restrict__ ge, int nelmt, const double* __restrict__ pold,
    const double* __restrict__ z, int combine, double* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ pos) {
  if (G && G->all_done) return;
  const int lane = threadIdx.x & 31;
  const int w0 = blockIdx.x * APPLY_WARPS + (threadIdx.x >> 5);
  const double beta = combine ? cs[0].beta : 0.0;
  for (int e = w0; e < nelmt; e += gridDim.x * APPLY_WARPS) {
    const int* g = ge + (size_t)e * NEDOF;
    int g0 = g[lane], g1 = g[lane + 32], g2 = lane < 17 ? g[lane + 64] : 0;
    double p0 = pold[g0], p1 = pold[g1], p2 = lane < 17 ? pold[g2] : 0.0;
    if (combine) {
      p0 = pdir(beta, p0, z[g0]);
      p1 = pdir(beta, p1, z[g1]);
      p2 = lane < 17 ? pdir(beta, p2, z[g2]) : 0.0;
    }
    const double* k = K + (size_t)e * NEDOF * NEDOF;
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
#pragma unroll
    for (int c = 0; c < NEDOF; ++c) {
      double src = c < 32 ? p0 : (c < 64 ? p1 : p2);
      double pc = __shfl_sync(FULL, src, c & 31);
      const double* col = k + (size_t)c * NEDOF;
      y0 = fma(__ldcs(col + lane), pc, y0);
      y1 = fma(__ldcs(col + lane + 32), pc, y1);
      if (lane < 17) y2 = fma(__ldcs(col + lane + 64), pc, y2);
    }
    // row r = 3a + d goes to the gather position of slot (e, a)
    const int* pe = pos + (size_t)e * NGLL;
    int q0 = pe[lane / 3], q1 = pe[(lane + 32) / 3];
    if (q0 >= 0) Y[(size_t)q0 * 3 + lane % 3] = y0;
    if (q1 >= 0) Y[(size_t)q1 * 3 + (lane + 32) % 3] = y1;
    if (lane < 17) {
      int q2 = pe[(lane + 64) / 3];
      if (q2 >= 0) Y[(size_t)q2 * 3 + (lane + 64) % 3] = y2;
    }
  }
}

// Sparse symmetric layout, KR right-hand sides (vectors are [dof][KR]).
// One warp per element: K_e (KS_STRIDE values) and p_e (81*KR) are staged in
// shared memory with 16-byte streaming loads, then lane n < 27 forms the
// three rows of node n from its 19 coupled node blocks.  The lane table nbr
// gives, per (n, s), the coupled node m, the block offset and whether the
// stored block is (n,m) (row-major access) or (m,n) (transposed access).
template <typename V, int KR>
__global__ void __launch_bounds__(APPLY_WARPS * 32) k_apply_sparse(
    const V* __restrict__ Ks, const int* __restrict__ ge, int nelmt, const V* __restrict__ pold,
    const V* __restrict__ z, int combine, V* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ nbr_g, const int* __restrict__ pos) {
  if (G && G->all_done) return;
  extern __shared__ __align__(128) unsigned char smem[];
  int* nbr = (int*)smem;                                   // 27*19 ints (2064 B incl. pad)
  V* wbase = (V*)(smem + 2064);
  constexpr int WSTRIDE = KS_STRIDE + ((NEDOF * KR + 3) & ~3);  // keeps every warp region 16-byte aligned
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  V* ks = wbase + warp * WSTRIDE;
  V* ps = ks + KS_STRIDE;
  for (int t = threadIdx.x; t < NGLL * KS_NBR; t += blockDim.x) nbr[t] = nbr_g[t];
  V beta[KR];
#pragma unroll
  for (int j = 0; j < KR; ++j) beta[j] = (V)(combine ? cs[j].beta : 0.0);
  __syncthreads();
  constexpr int NV = KS_STRIDE * (int)sizeof(V) / 16;
  for (int e = blockIdx.x * APPLY_WARPS + warp; e < nelmt; e += gridDim.x * APPLY_WARPS) {
    const float4* src = reinterpret_cast<const float4*>(Ks + (size_t)e * KS_STRIDE);
    float4* dst = reinterpret_cast<float4*>(ks);
#pragma unroll 4
    for (int q = lane; q < NV; q += 32) dst[q] = __ldcs(src + q);
    if (lane < NGLL) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int g = ge[(size_t)e * NEDOF + 3 * lane + d];
#pragma unroll
        for (int j = 0; j < KR; ++j) {
          V pv = pold[(size_t)g * KR + j];
          if (combine) pv = pdir(beta[j], pv, z[(size_t)g * KR + j]);
          ps[(3 * lane + d) * KR + j] = pv;
        }
      }
    }
    __syncwarp();
    if (lane < NGLL) {
      V acc[3][KR];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < KR; ++j) acc[c][j] = (V)0;
      const int* tb = nbr + lane * KS_NBR;
#pragma unroll 1
      for (int s = 0; s < KS_NBR; ++s) {
        int pk = tb[s];
        int m = pk & 31, kind = (pk >> 5) & 3, off = pk >> 8;
        int sc = (kind == 2) ? 1 : 3, sd = (kind == 2) ? 3 : 1;
        const V* kb = ks + off;
        const V* pm = ps + 3 * m * KR;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            V kv = kb[c * sc + d * sd];
#pragma unroll
            for (int j = 0; j < KR; ++j) acc[c][j] = fmav<V>(kv, pm[d * KR + j], acc[c][j]);
          }
        }
      }
      const int q = pos[(size_t)e * NGLL + lane];
      if (q >= 0) storev3<V, KR>(Y + (size_t)q * 3 * KR, acc);
    }
    __syncwarp();
  }
}

// ---- TMA-staged variant: 1D bulk copies (cp.async.bulk) of each element's
// matrix into a two-stage per-warp ring, completion tracked by mbarriers.
// Lane 0 issues the copy of the warp's next element before the warp computes
// the current one, so the HBM stream overlaps the shared-memory matvec.
// Every wait is bounded: on timeout the kernel records the fault in *err and
// the warp stops after draining its own copies (also bounded).

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// returns false if the phase did not complete within the bound
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int tries = 0; tries < (1 << 22); ++tries) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

template <typename V, int KR>
__global__ void __launch_bounds__(APPLY_WARPS * 32) k_apply_sparse_tma(
    const V* __restrict__ Ks, const int* __restrict__ ge, int nelmt, const V* __restrict__ pold,
    const V* __restrict__ z, int combine, V* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ nbr_g, const int* __restrict__ pos,
    int* __restrict__ err) {
  if (G && G->all_done) return;
  extern __shared__ __align__(128) unsigned char smem[];
  // p tile: one row of 3*KR values per node, padded so that node rows start
  // 4 banks apart modulo 32 (a period-8 bank pattern for the 16-byte reads)
  constexpr int PROW = 3 * KR + (KR >= 8 ? 4 : 0);
  constexpr int PST = (NGLL * PROW + 3) & ~3;
  constexpr int WSTRIDE = 2 * KS_STRIDE + PST;     // two K stages + the p tile
  constexpr unsigned KBYTES = KS_STRIDE * sizeof(V);
  int* nbr = (int*)smem;                           // 27*19 ints
  uint64_t* bars = (uint64_t*)(smem + 2944);       // 2 mbarriers per warp
  V* wbase = (V*)(smem + 3072);                    // 128-byte aligned base
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  V* kbuf0 = wbase + (size_t)warp * WSTRIDE;
  V* kbuf1 = kbuf0 + KS_STRIDE;
  V* ps = kbuf1 + KS_STRIDE;
  uint64_t* bar = bars + 2 * warp;
  for (int t = threadIdx.x; t < NGLL * KS_NBR; t += blockDim.x) nbr[t] = nbr_g[t];
  if (lane == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  V beta[KR];
#pragma unroll
  for (int j = 0; j < KR; ++j) beta[j] = (V)(combine ? cs[j].beta : 0.0);
  __syncthreads();
  const int stride = gridDim.x * APPLY_WARPS;
  int e = blockIdx.x * APPLY_WARPS + warp;
  if (e < nelmt && lane == 0) bulk_load(kbuf0, Ks + (size_t)e * KS_STRIDE, KBYTES, bar);
  int issued = (e < nelmt) ? 1 : 0, waited = 0;
  for (int i = 0; e < nelmt; ++i, e += stride) {
    const int en = e + stride;
    V* kcur = (i & 1) ? kbuf1 : kbuf0;
    if (en < nelmt && lane == 0) {
      V* knext = (i & 1) ? kbuf0 : kbuf1;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_load(knext, Ks + (size_t)en * KS_STRIDE, KBYTES, bar + ((i + 1) & 1));
      ++issued;
    }
    if (lane < NGLL) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int g = ge[(size_t)e * NEDOF + 3 * lane + d];
        V pv[KR];
        loadv<V, KR>(pold + (size_t)g * KR, pv);
        if (combine) {
          V zv[KR];
          loadv<V, KR>(z + (size_t)g * KR, zv);
#pragma unroll
          for (int j = 0; j < KR; ++j) pv[j] = pdir(beta[j], pv[j], zv[j]);
        }
#pragma unroll
        for (int j = 0; j < KR; ++j) ps[lane * PROW + d * KR + j] = pv[j];
      }
    }
    bool ok = mbar_wait(bar + (i & 1), (unsigned)((i >> 1) & 1));
    ++waited;
    if (!ok) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
    __syncwarp();
    if (lane < NGLL) {
      V acc[3][KR];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < KR; ++j) acc[c][j] = (V)0;
      const int* tb = nbr + lane * KS_NBR;
      if constexpr (std::is_same<V, float>::value && KR % 4 == 0) {
        // packed FP32x2 FMAs: two right-hand sides per instruction (p rows
        // are read as 16-byte vectors, so KR must be a multiple of 4)
        float2 acc2[3][KR / 2];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int q = 0; q < KR / 2; ++q) acc2[c][q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int s = 0; s < KS_NBR; ++s) {
          int pk = tb[s];
          int m = pk & 31, kind = (pk >> 5) & 3, off = pk >> 8;
          int sc = (kind == 2) ? 1 : 3, sd = (kind == 2) ? 3 : 1;
          const V* kb = kcur + off;
          const V* pm = ps + m * PROW;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            float2 pv2[KR / 2];
#pragma unroll
            for (int q = 0; q < KR / 4; ++q) {
              float4 t = reinterpret_cast<const float4*>(pm + d * KR)[q];
              pv2[2 * q] = make_float2(t.x, t.y);
              pv2[2 * q + 1] = make_float2(t.z, t.w);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float kv = kb[c * sc + d * sd];
              const float2 kk = make_float2(kv, kv);
#pragma unroll
              for (int q = 0; q < KR / 2; ++q) acc2[c][q] = __ffma2_rn(kk, pv2[q], acc2[c][q]);
            }
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int q = 0; q < KR / 2; ++q) { acc[c][2 * q] = acc2[c][q].x; acc[c][2 * q + 1] = acc2[c][q].y; }
      } else {
#pragma unroll
        for (int s = 0; s < KS_NBR; ++s) {
          int pk = tb[s];
          int m = pk & 31, kind = (pk >> 5) & 3, off = pk >> 8;
          int sc = (kind == 2) ? 1 : 3, sd = (kind == 2) ? 3 : 1;
          const V* kb = kcur + off;
          const V* pm = ps + m * PROW;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            V pv[KR];
            loadv<V, KR>(pm + d * KR, pv);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              V kv = kb[c * sc + d * sd];
#pragma unroll
              for (int j = 0; j < KR; ++j) acc[c][j] = fmav<V>(kv, pv[j], acc[c][j]);
            }
          }
        }
      }
      const int q = pos[(size_t)e * NGLL + lane];
      if (q >= 0) storev3<V, KR>(Y + (size_t)q * 3 * KR, acc);
    }
    __syncwarp();
  }
  // drain copies still in flight after an early stop (bounded)
  for (int i = waited; i < issued; ++i) mbar_wait(bar + (i & 1), (unsigned)((i >> 1) & 1));
}

template <typename V, int KR>
static size_t apply_tma_smem() {
  constexpr int PROW = 3 * KR + (KR >= 8 ? 4 : 0);
  return 3072 + (size_t)APPLY_WARPS * (2 * KS_STRIDE + ((NGLL * PROW + 3) & ~3)) * sizeof(V);
}

template <typename V, int KR>
static size_t apply_sparse_smem() {
  return 2064 + (size_t)APPLY_WARPS * (KS_STRIDE + ((NEDOF * KR + 3) & ~3)) * sizeof(V);
}

template <typename V, int KR>
void pcg_apply(int dense, const void* K, const int* ge, int nelmt, const V* p_old, const V* z, int combine, V* Y,
               const ColState* cs, const PcgGlobal* G, const int* d_nbr, const int* pos, int* err, cudaStream_t s) {
  if (nelmt <= 0) return;
  int blocks = (nelmt + APPLY_WARPS - 1) / APPLY_WARPS;
  if (dense == 2) {
    if constexpr (std::is_same<V, float>::value)
      SG_LAUNCH launch_apply_mf<KR>((const float*)K, ge, nelmt, p_old, z, combine, Y, cs, G, pos, s);
    return;
  }
  if (dense) {
    if constexpr (std::is_same<V, double>::value && KR == 1)
      SG_LAUNCH k_apply_dense64<<<blocks, APPLY_WARPS * 32, 0, s>>>((const double*)K, ge, nelmt, p_old, z, combine, Y, cs, G,
                                                                    pos);
    return;
  }
  if constexpr (std::is_same<V, float>::value && (KR == 8 || KR == 16)) {
    if (g_apply_variant == 2) {
      SG_LAUNCH launch_apply_tc<KR>((const float*)K, ge, nelmt, p_old, z, combine, Y, cs, G, g_entry_dev, pos, err, s);
      return;
    }
    if (g_apply_variant >= 3) {
      SG_LAUNCH launch_apply_lanes<KR>((const float*)K, ge, nelmt, p_old, z, combine, Y, cs, G, pos, err, s);
      return;
    }
  }
  if (g_apply_variant >= 1) {
    size_t sm = apply_tma_smem<V, KR>();
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_apply_sparse_tma<V, KR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      attr = true;
    }
    // persistent-style grid: each warp walks a strided list of elements
    int per_sm = (int)(200 * 1024 / sm);
    if (per_sm < 1) per_sm = 1;
    int grid = std::min(blocks, 152 * per_sm);
    SG_LAUNCH k_apply_sparse_tma<V, KR><<<grid, APPLY_WARPS * 32, sm, s>>>((const V*)K, ge, nelmt, p_old, z, combine, Y, cs,
                                                                 G, d_nbr, pos, err);
    return;
  }
  size_t sm = apply_sparse_smem<V, KR>();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_apply_sparse<V, KR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  SG_LAUNCH k_apply_sparse<V, KR><<<blocks, APPLY_WARPS * 32, sm, s>>>((const V*)K, ge, nelmt, p_old, z, combine, Y, cs, G,
                                                               d_nbr, pos);
}

// ---------------------------------------------------------------------------
// Gather: kp(dof) = sum over the node's element slots, in element order, of Y.
// mode 0: plain (kp only); mode 1: PCG iteration -- also p = z + beta*p for
// the node's dofs and the p.kp partial; the last block forms alpha = rz/p.kp.
// ---------------------------------------------------------------------------
// Each warp takes 32 consecutive groups; their element slots are one
// contiguous run of Y (the producers wrote slot s at position s), which the
// warp copies into shared memory with coalesced 16-byte loads before each lane
// sums its own group's slots in order.  A run longer than the buffer is read
// directly from global memory.
constexpr int GATHER_WARPS = RED_THREADS / 32;

// Grid of a PCG kernel with a last-block reduction: enough blocks for `per`
// items each, at most `cap`.  Small problems get few blocks, so the last
// block sums few partials; the grid depends only on the problem size, so the
// reduction order (and the result) stays fixed for a given problem.
static inline int red_grid(size_t items, size_t per, int cap) {
  size_t g = (items + per - 1) / per;
  return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)cap));
}

template <typename V, int KR>
struct GatherBuf {
  static constexpr int ROW = 3 * KR;                                    // values per slot
  // slots per warp buffer: 32 groups hold ~108 slots on average (27/8 per node)
  static constexpr int CAP_BYTES = (20480 / (ROW * (int)sizeof(V))) & ~1;
  static constexpr int CAP = CAP_BYTES < 128 ? CAP_BYTES : 128;
  static constexpr size_t SMEM = (size_t)GATHER_WARPS * CAP * ROW * sizeof(V);
};

template <typename V, int KR>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_gather(
    const int* __restrict__ ptr, const int* __restrict__ ent, const int* __restrict__ dof, int ng,
    const V* __restrict__ Y, V* __restrict__ kp, V* __restrict__ p, const V* __restrict__ z, int mode,
    ColState* __restrict__ cs, PcgGlobal* __restrict__ G, double* __restrict__ part) {
  if (G->all_done) return;
  constexpr int ROW = GatherBuf<V, KR>::ROW, CAP = GatherBuf<V, KR>::CAP;
  extern __shared__ __align__(128) unsigned char gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  DotAcc<V> dacc[KR];
  bool live[KR];
  V beta[KR];
#pragma unroll
  for (int j = 0; j < KR; ++j) {
    live[j] = cs[j].active && !cs[j].done;
    beta[j] = (V)cs[j].beta;
  }
  V* buf = reinterpret_cast<V*>(gsm) + (size_t)warp * CAP * ROW;
  for (int g0 = (blockIdx.x * GATHER_WARPS + warp) * 32; g0 < ng; g0 += gridDim.x * GATHER_WARPS * 32) {
    const int g = g0 + lane;
    const int gend = min(g0 + 32, ng);
    const int s0 = ptr[g0], s1 = ptr[gend];
    const int a = g < ng ? ptr[g] : s1, b = g < ng ? ptr[g + 1] : s1;
    const bool staged = (s1 - s0) <= CAP;
    if (staged) {
      const size_t base = (size_t)s0 * ROW;
      const int nval = (s1 - s0) * ROW;
      if constexpr ((ROW * sizeof(V)) % 16 == 0) {
        const float4* src = reinterpret_cast<const float4*>(Y + base);
        float4* dst = reinterpret_cast<float4*>(buf);
        const int n4 = nval * (int)sizeof(V) / 16;
        for (int q = lane; q < n4; q += 32) dst[q] = __ldcs(src + q);
      } else {
        for (int q = lane; q < nval; q += 32) buf[q] = Y[base + q];
      }
    }
    __syncwarp();
    // one dof of the node at a time keeps the accumulators to KR registers
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
      V acc[KR];
#pragma unroll
      for (int j = 0; j < KR; ++j) acc[j] = (V)0;
      for (int s = a; s < b; ++s) {
        const V* y = (staged ? buf + (size_t)(s - s0) * ROW : Y + (size_t)s * ROW) + d * KR;
        V yv[KR];
        loadv<V, KR>(y, yv);
#pragma unroll
        for (int j = 0; j < KR; ++j) acc[j] = acc[j] + yv[j];
      }
      const int gd = g < ng ? dof[3 * g + d] : 0;
      if (!gd) continue;
      V* kpo = kp + (size_t)gd * KR;
      if (mode == 0) {
        storev<V, KR>(kpo, acc);
        continue;
      }
      V pv[KR], zv[KR];
      loadv<V, KR>(p + (size_t)gd * KR, pv);
      loadv<V, KR>(z + (size_t)gd * KR, zv);
#pragma unroll
      for (int j = 0; j < KR; ++j) {
        if (live[j]) {
          pv[j] = pdir(beta[j], pv[j], zv[j]);
          dacc[j].add(pv[j], acc[j]);
        }
      }
      storev<V, KR>(p + (size_t)gd * KR, pv);
      storev<V, KR>(kpo, acc);
    }
    __syncwarp();
  }
  if (mode == 0) return;
  __shared__ double sred[RED_THREADS / 32][KR];
#pragma unroll
  for (int j = 0; j < KR; ++j) {
    double v = dacc[j].value();
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0) sred[warp][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < KR) {
    double v = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) v += sred[w][threadIdx.x];
    part[(size_t)blockIdx.x * KR + threadIdx.x] = v;
  }
  if (last_block(&G->cntB)) {
    // all threads: thread t sums blocks t/KR, t/KR + RED_THREADS/KR, ... of column t%KR in order
    __shared__ double sfin[RED_THREADS];
    double v = 0.0;
    for (int idx = threadIdx.x; idx < (int)gridDim.x * KR; idx += RED_THREADS) v += __ldcg(part + idx);
    sfin[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < KR) {
      int j = threadIdx.x;
      double s = 0.0;
      for (int t = j; t < RED_THREADS; t += KR) s += sfin[t];
      if (cs[j].active && !cs[j].done) cs[j].alpha = cs[j].rz / s;
    }
    if (threadIdx.x == 0) G->cntB = 0;
  }
}

// Row-cooperative gather for FP32 with KR = 4, 8 or 16: a node's slot rows
// (3*KR floats) are read by LPN = 3*KR/4 lanes, one 16-byte piece each, so a
// warp's loads are coalesced runs of Y and no shared memory is needed.  Lane
// (node, q) sums piece q over the node's slots in element order -- the same
// additions in the same order as the staged gather, so kp and p are bitwise
// equal to it; the p.kp partials are compensated sums over the lane's four
// columns, reduced in a fixed order.
int g_gather_variant = 1;   // 0 = staged gather for every case
constexpr int GATHER_ROWS_BLOCKS = 152 * 4;   // one wave: four resident CTAs per SM at 64 registers
static_assert(GATHER_ROWS_BLOCKS * 16 <= NPART * 16 * 4, "p.kp partials fit the partial buffer");
void set_gather_variant(int v) { g_gather_variant = v; }

template <int KR>
__global__ void __launch_bounds__(RED_THREADS, 4) k_pcg_gather_rows(
    const int* __restrict__ ptr, const int* __restrict__ dof, int ng, const float* __restrict__ Y,
    float* __restrict__ kp, float* __restrict__ p, const float* __restrict__ z, int mode, ColState* __restrict__ cs,
    PcgGlobal* __restrict__ G, double* __restrict__ part) {
  if (G->all_done) return;
  constexpr int QPD = KR / 4;      // 16-byte pieces per dof row
  constexpr int LPN = 3 * QPD;     // lanes per node
  constexpr int NPW = 32 / LPN;    // nodes per warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nl = lane / LPN, q = lane - nl * LPN;
  const int d = q / QPD, c0 = 4 * (q - d * QPD);
  const bool act = nl < NPW;
  DotAcc<float> dacc[4];
  bool live[4];
  float beta[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int j = act ? c0 + k : 0;
    live[k] = act && cs[j].active && !cs[j].done;
    beta[k] = (float)cs[j].beta;
  }
  const float4* yq = reinterpret_cast<const float4*>(Y) + q;
  const int wstride = gridDim.x * GATHER_WARPS * NPW;
  for (int g0 = (blockIdx.x * GATHER_WARPS + warp) * NPW; g0 < ng; g0 += wstride) {
    const int g = g0 + nl;
    if (!act || g >= ng) continue;
    const int a = ptr[g], b = ptr[g + 1];
    const int gd = dof[3 * g + d];
    // the p and z rows do not depend on the sums: their loads go out with the
    // first slot loads (two dependent trips per node instead of three)
    float4* pp = reinterpret_cast<float4*>(p + (size_t)gd * KR + c0);
    float4 pv = make_float4(0.f, 0.f, 0.f, 0.f), zv = pv;
    if (mode != 0 && gd) {
      pv = *pp;
      zv = *reinterpret_cast<const float4*>(z + (size_t)gd * KR + c0);
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    // up to four slots in flight at once, summed in slot order
    float4 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (a + k < b) v[k] = __ldcs(yq + (size_t)(a + k) * LPN);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (a + k < b) {
        acc.x = acc.x + v[k].x;
        acc.y = acc.y + v[k].y;
        acc.z = acc.z + v[k].z;
        acc.w = acc.w + v[k].w;
      }
    for (int sl = a + 4; sl < b; ++sl) {
      const float4 w = __ldcs(yq + (size_t)sl * LPN);
      acc.x = acc.x + w.x;
      acc.y = acc.y + w.y;
      acc.z = acc.z + w.z;
      acc.w = acc.w + w.w;
    }
    if (!gd) continue;
    float4* kpo = reinterpret_cast<float4*>(kp + (size_t)gd * KR + c0);
    if (mode == 0) {
      *kpo = acc;
      continue;
    }
    if (live[0]) { pv.x = pdir(beta[0], pv.x, zv.x); dacc[0].add(pv.x, acc.x); }
    if (live[1]) { pv.y = pdir(beta[1], pv.y, zv.y); dacc[1].add(pv.y, acc.y); }
    if (live[2]) { pv.z = pdir(beta[2], pv.z, zv.z); dacc[2].add(pv.z, acc.z); }
    if (live[3]) { pv.w = pdir(beta[3], pv.w, zv.w); dacc[3].add(pv.w, acc.w); }
    *pp = pv;
    *kpo = acc;
  }
  if (mode == 0) return;
  __shared__ double sred[RED_THREADS / 32][KR];
  double mine[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) mine[k] = act ? dacc[k].value() : 0.0;
#pragma unroll
  for (int j = 0; j < KR; ++j) {
    double v = (act && (j >> 2) == (c0 >> 2)) ? mine[j & 3] : 0.0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0) sred[warp][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < KR) {
    double v = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) v += sred[w][threadIdx.x];
    part[(size_t)blockIdx.x * KR + threadIdx.x] = v;
  }
  if (last_block(&G->cntB)) {
    __shared__ double sfin[RED_THREADS];
    double v = 0.0;
    for (int idx = threadIdx.x; idx < (int)gridDim.x * KR; idx += RED_THREADS) v += __ldcg(part + idx);
    sfin[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < KR) {
      int j = threadIdx.x;
      double t = 0.0;
      for (int u = j; u < RED_THREADS; u += KR) t += sfin[u];
      if (cs[j].active && !cs[j].done) cs[j].alpha = cs[j].rz / t;
    }
    if (threadIdx.x == 0) G->cntB = 0;
  }
}

// Fused FP32 PCG step for 8 or 16 columns (residual-reduction mode): with
// the element apply forming p_k = beta_k p_{k-1} + D (r_{k-1} - alpha_{k-1}
// kp_{k-1}) on the fly, one kernel per step does the rest of src/solver.f90:
// 53-73 for every free dof row (node, dof, four columns):
//   q = kp_k   = sum of the row's element products in element order
//   u += alpha_{k-1} p_{k-1},  r_k = r_{k-1} - alpha_{k-1} kp_{k-1},  z_k = D r_k,
//   p_k = beta_k p_{k-1} + z_k   (bitwise the p_k of the apply)
// and the partial sums p_k.q, q.z_k, q.(D q), r_k.r_k, max|p_k| and
// gamma_k = r_k.z_k.  The last block stops a column when r_k.r_k <= tol^2
// r_0.r_0 (k-1 completed steps); otherwise alpha_k = gamma_k / p_k.q and,
// without forming r_{k+1}, one step of the recurrence
//   gamma_{k+1} = gamma_k - 2 alpha_k q.z_k + alpha_k^2 q.(D q),
//   beta_{k+1} = gamma_{k+1} / gamma_k.
// gamma_k itself is summed directly every step: carried from step to step,
// the recurrence keeps the absolute rounding error of the largest gamma it
// has seen, which swamps gamma once the FP32 residual has dropped by 1e3
// (on the layered 3D slope it turned negative within 30 steps).  A single
// step of it errs by about eps_f32 * sqrt(gamma_k / gamma_{k+1}) relative.
// So an iteration is two kernels (apply, this) instead of three, and u, r,
// z and kp make one trip through HBM fewer.  The dots use the compensated
// FP32 sums of the other kernels; r.r only feeds the stop test and is summed
// plainly.
constexpr int GU_NQ = 8;                 // partial quantities per column (6 used)
constexpr int GU_USED = 6;
constexpr int GU_BLOCKS = 152 * 2;       // two resident CTAs per SM (128 registers)

template <int KR>
__global__ void __launch_bounds__(RED_THREADS, 2) k_pcg_gather_update(
    const int* __restrict__ ptr, const int* __restrict__ dof, int ng, const float* __restrict__ Y,
    float* __restrict__ kp, float* __restrict__ p, float* __restrict__ r, float* __restrict__ u,
    const float* __restrict__ dinv, ColState* __restrict__ cs, PcgGlobal* __restrict__ G, double* __restrict__ part) {
  if (G->all_done) return;
  constexpr int QPD = KR / 4;      // 16-byte pieces per dof row
  constexpr int LPN = 3 * QPD;     // lanes per node
  constexpr int NPW = 32 / LPN;    // nodes per warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nl = lane / LPN, q = lane - nl * LPN;
  const int d = q / QPD, c0 = 4 * (q - d * QPD);
  const bool act = nl < NPW;
  bool live[4];
  float alpha[4], beta[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int j = act ? c0 + k : 0;
    live[k] = act && cs[j].active && !cs[j].done;
    alpha[k] = (float)cs[j].alpha;
    beta[k] = (float)cs[j].beta;
  }
  DotAcc<float> sd[4], sa[4], sb[4], sg[4];
  float srr[4] = {0.f, 0.f, 0.f, 0.f}, smp[4] = {0.f, 0.f, 0.f, 0.f};
  const float4* yq = reinterpret_cast<const float4*>(Y) + q;
  const int wstride = gridDim.x * GATHER_WARPS * NPW;
  for (int g0 = (blockIdx.x * GATHER_WARPS + warp) * NPW; g0 < ng; g0 += wstride) {
    const int g = g0 + nl;
    if (!act || g >= ng) continue;
    const int a = ptr[g], b = ptr[g + 1];
    const int gd = dof[3 * g + d];
    const size_t o = (size_t)gd * KR + c0;
    float4 pv = make_float4(0.f, 0.f, 0.f, 0.f), rv = pv, kv = pv, uv = pv;
    float dv = 0.f;
    if (gd) {
      pv = *reinterpret_cast<const float4*>(p + o);
      rv = *reinterpret_cast<const float4*>(r + o);
      kv = *reinterpret_cast<const float4*>(kp + o);
      uv = *reinterpret_cast<const float4*>(u + o);
      dv = dinv[gd];
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (a + k < b) v[k] = __ldcs(yq + (size_t)(a + k) * LPN);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (a + k < b) {
        acc.x = acc.x + v[k].x;
        acc.y = acc.y + v[k].y;
        acc.z = acc.z + v[k].z;
        acc.w = acc.w + v[k].w;
      }
    for (int sl = a + 4; sl < b; ++sl) {
      const float4 w = __ldcs(yq + (size_t)sl * LPN);
      acc.x = acc.x + w.x;
      acc.y = acc.y + w.y;
      acc.z = acc.z + w.z;
      acc.w = acc.w + w.w;
    }
    if (!gd) continue;
    float pa[4] = {pv.x, pv.y, pv.z, pv.w}, ra[4] = {rv.x, rv.y, rv.z, rv.w};
    float ka[4] = {kv.x, kv.y, kv.z, kv.w}, ua[4] = {uv.x, uv.y, uv.z, uv.w};
    const float qa[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!live[k]) continue;          // stopped or inactive columns keep u, r and p
      const float un = fmaf(alpha[k], pa[k], ua[k]);
      const float rn = fmaf(-alpha[k], ka[k], ra[k]);
      const float zn = dv * rn;
      const float pn = fmaf(beta[k], pa[k], zn);
      sd[k].add(pn, qa[k]);
      sa[k].add(qa[k], zn);
      sg[k].add(rn, zn);
      sb[k].add(qa[k], dv * qa[k]);
      srr[k] = fmaf(rn, rn, srr[k]);
      smp[k] = fmaxf(smp[k], fabsf(pn));
      ua[k] = un; ra[k] = rn; pa[k] = pn;
    }
    *reinterpret_cast<float4*>(u + o) = make_float4(ua[0], ua[1], ua[2], ua[3]);
    *reinterpret_cast<float4*>(r + o) = make_float4(ra[0], ra[1], ra[2], ra[3]);
    *reinterpret_cast<float4*>(p + o) = make_float4(pa[0], pa[1], pa[2], pa[3]);
    *reinterpret_cast<float4*>(kp + o) = acc;
  }
  // block partials: [block][column][GU_NQ] = p.q, q.z, q.Dq, r.r, max|p|, r.z
  __shared__ double sred[RED_THREADS / 32][KR][GU_USED];
  auto mine = [&](int k, int qq) -> double {
    if (!(act && live[k])) return 0.0;
    return qq == 0 ? sd[k].value() : qq == 1 ? sa[k].value() : qq == 2 ? sb[k].value()
                   : qq == 3 ? (double)srr[k] : qq == 4 ? (double)smp[k] : sg[k].value();
  };
#pragma unroll
  for (int j = 0; j < KR; ++j) {
    const bool own = act && (j >> 2) == (c0 >> 2);
#pragma unroll
    for (int qq = 0; qq < GU_USED; ++qq) {
      double v = own ? mine(j & 3, qq) : 0.0;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const double w = __shfl_xor_sync(FULL, v, o);
        v = (qq == 4) ? fmax(v, w) : v + w;
      }
      if (lane == 0) sred[warp][j][qq] = v;
    }
  }
  __syncthreads();
  // all GU_NQ slots are written (the unused ones as zero), so the last block
  // never reads partial memory that no block has written
  if (threadIdx.x < KR * GU_NQ) {
    const int j = threadIdx.x / GU_NQ, qq = threadIdx.x % GU_NQ;
    double v = 0.0;
    if (qq < GU_USED)
      for (int w = 0; w < RED_THREADS / 32; ++w) v = (qq == 4) ? fmax(v, sred[w][j][qq]) : v + sred[w][j][qq];
    part[((size_t)blockIdx.x * KR + j) * GU_NQ + qq] = v;
  }
  if (!last_block(&G->cntB)) return;
  // fixed-order reduction of the block partials: thread t owns quantity t % GU_NQ
  __shared__ double sfin[RED_THREADS];
  __shared__ int s_alldone;
  {
    constexpr int NQ = GU_NQ * KR;
    static_assert(RED_THREADS % NQ == 0, "a thread keeps one quantity");
    const int qq = threadIdx.x % GU_NQ;
    double v = 0.0;
    for (int idx = threadIdx.x; idx < (int)gridDim.x * NQ; idx += RED_THREADS) {
      const double x = __ldcg(part + idx);
      v = (qq == 4) ? fmax(v, x) : v + x;
    }
    sfin[threadIdx.x] = v;
  }
  if (threadIdx.x == 0) s_alldone = 1;
  __syncthreads();
  const int it = G->it + 1;
  if (threadIdx.x < KR) {
    constexpr int NQ = GU_NQ * KR;
    const int jj = threadIdx.x;
    ColState& c = cs[jj];
    double pq = 0.0, qz = 0.0, qdq = 0.0, rr = 0.0, mp = 0.0, rz = 0.0;
    for (int t = jj * GU_NQ; t < RED_THREADS; t += NQ) {
      pq += sfin[t]; qz += sfin[t + 1]; qdq += sfin[t + 2]; rr += sfin[t + 3]; mp = fmax(mp, sfin[t + 4]);
      rz += sfin[t + 5];
    }
    if (c.active && !c.done) {
      c.rr = rr;
      if (rr <= c.tol * c.tol * c.rr0) {
        // alpha, maxp and rz (the one-step recurrence value that formed
        // beta of the direction in p) stay those of the last step taken
        c.done = 1; c.iters = it - 1;
      } else if (it - 1 >= G->maxiter) {
        c.done = 1; c.failed = 1; c.iters = G->maxiter + 1;
      } else {
        const double al = rz / pq;
        const double gn = rz - 2.0 * al * qz + al * al * qdq;
        c.alpha = al;
        // a non-positive one-step value (rounding at the end of a solve)
        // restarts the direction instead of reversing it
        c.beta = gn > 0.0 ? gn / rz : 0.0;
        c.rz = gn > 0.0 ? gn : rz;
        c.maxp = mp;
      }
    }
    if (jj < G->kcols && c.active && !c.done) atomicAnd(&s_alldone, 0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    G->it = it;
    G->all_done = s_alldone;
    G->cntB = 0;
  }
}

template <int KR>
void pcg_gather_update(const GatherTopo& T, const float* Y, float* kp, float* p, float* r, float* u,
                       const float* dinv, ColState* cs, PcgGlobal* G, double* part, cudaStream_t s) {
  constexpr int NPB = GATHER_WARPS * (32 / (3 * KR / 4));       // nodes per block and pass
  constexpr int CAP_PART = NPART * 16 * 4 / (GU_NQ * KR);       // blocks whose partials fit
  constexpr int CAP = CAP_PART < GU_BLOCKS ? CAP_PART : GU_BLOCKS;
  SG_LAUNCH k_pcg_gather_update<KR><<<red_grid(T.ngroups, NPB * 4, CAP), RED_THREADS, 0, s>>>(
      T.d_ptr, T.d_dof, T.ngroups, Y, kp, p, r, u, dinv, cs, G, part);
}
template void pcg_gather_update<8>(const GatherTopo&, const float*, float*, float*, float*, float*, const float*,
                                   ColState*, PcgGlobal*, double*, cudaStream_t);
template void pcg_gather_update<16>(const GatherTopo&, const float*, float*, float*, float*, float*, const float*,
                                    ColState*, PcgGlobal*, double*, cudaStream_t);

// End of a fused solve.  A column that stopped after k steps holds r_k and
// the direction of step k+1, p_{k+1} = beta_{k+1} p_k + D r_k, with
// rz = r_k.z_k.  Taking D r_k off leaves beta_{k+1} p_k, so that a solve
// that continues the direction (keep_dir: p = (r.z_new / rz) p_old + z_new)
// forms (r.z_new / r_{k-1}.z_{k-1}) p_k + z_new, the continuation of the
// three-kernel iteration.  Columns that did not take part keep their p.
template <int KR>
__global__ void __launch_bounds__(RED_THREADS) k_fused_dir_restore(int n1, float* __restrict__ p,
                                                                 const float* __restrict__ r,
                                                                 const float* __restrict__ dinv,
                                                                 const ColState* __restrict__ cs) {
  const int j = threadIdx.x & (KR - 1);
  if (!cs[j].active) return;
  const size_t n = (size_t)n1 * KR;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = p[i] - dinv[i / KR] * r[i];
}

template <int KR>
void fused_dir_restore(int n1, float* p, const float* r, const float* dinv, const ColState* cs, cudaStream_t s) {
  SG_LAUNCH k_fused_dir_restore<KR><<<red_grid((size_t)n1 * KR, RED_THREADS * 4, 152 * 8), RED_THREADS, 0, s>>>(
      n1, p, r, dinv, cs);
}
template void fused_dir_restore<8>(int, float*, const float*, const float*, const ColState*, cudaStream_t);
template void fused_dir_restore<16>(int, float*, const float*, const float*, const ColState*, cudaStream_t);

// Off by default: on the 192k-element slope with 8 trials the fused step took
// 0.798 + 0.399 ms against 0.717 + 0.231 + 0.207 ms for the three kernels
// (the apply's direction then gathers r, kp and D besides p).
bool fused_pcg_enabled() {
  static const bool on = getenv("SG_FUSED") && atoi(getenv("SG_FUSED")) == 1;
  return on;
}
bool apply_uses_lanes(int dense, int KR) { return dense == 0 && (KR == 8 || KR == 16) && g_apply_variant >= 3; }

template <typename V, int KR>
void pcg_gather(const GatherTopo& T, const V* Y, V* kp, V* p, const V* z, int mode, ColState* cs, PcgGlobal* G,
                double* part, cudaStream_t s) {
  if constexpr (std::is_same<V, float>::value && (KR == 4 || KR == 8 || KR == 16)) {
    if (g_gather_variant == 1) {
      // one wave of resident CTAs (the grid depends only on the problem size)
      constexpr int NPB = GATHER_WARPS * (32 / (3 * KR / 4));   // nodes per block and pass
      SG_LAUNCH k_pcg_gather_rows<KR><<<red_grid(T.ngroups, NPB * 4, GATHER_ROWS_BLOCKS), RED_THREADS, 0, s>>>(T.d_ptr, T.d_dof, T.ngroups, Y, kp, p, z, mode,
                                                                   cs, G, part);
      return;
    }
  }
  constexpr size_t sm = GatherBuf<V, KR>::SMEM;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_pcg_gather<V, KR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  SG_LAUNCH k_pcg_gather<V, KR><<<red_grid(T.ngroups, GATHER_WARPS * 32 * 2, NPART), RED_THREADS, sm, s>>>(T.d_ptr, T.d_ent, T.d_dof, T.ngroups, Y, kp, p, z, mode,
                                                              cs, G, part);
}

// Plain gather without PCG state: out = (accumulate ? out : 0) + sum Y.
template <typename V>
__global__ void k_gather_plain(const int* __restrict__ ptr, const int* __restrict__ ent, const int* __restrict__ dof,
                               int ng, int KR, const V* __restrict__ Y, V* __restrict__ out, int accumulate,
                               const int* __restrict__ colmask) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ng * KR) return;
  int g = t / KR, j = t - g * KR;
  if (colmask && !colmask[j]) return;
  V acc[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int gd = dof[3 * g + d];
    acc[d] = (accumulate && gd) ? out[(size_t)gd * KR + j] : (V)0;
  }
  for (int s = ptr[g]; s < ptr[g + 1]; ++s) {
    const V* y = Y + (size_t)s * 3 * KR;
#pragma unroll
    for (int d = 0; d < 3; ++d) acc[d] = acc[d] + y[d * KR + j];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int gd = dof[3 * g + d];
    if (gd) out[(size_t)gd * KR + j] = acc[d];
  }
}

template <typename V>
void launch_gather_plain(const GatherTopo& T, int KR, const V* Y, V* out, int accumulate, const int* colmask,
                         cudaStream_t s) {
  int n = T.ngroups * KR;
  if (n > 0) SG_LAUNCH k_gather_plain<V><<<(n + 255) / 256, 256, 0, s>>>(T.d_ptr, T.d_ent, T.d_dof, T.ngroups, KR, Y, out,
                                                               accumulate, colmask);
}

// ---------------------------------------------------------------------------
// PCG update (src/solver.f90:61-73).  init = 1: r = f - kp, z = D r, rz and
// |r|^2, beta = 0.  init = 0: u += alpha p, r -= alpha kp, z = D r and the
// partials max|p|, max|u|, r.z, |r|^2; the last block applies the stop test
// |alpha|*max|p|/max|u| <= tol (mode 0) or |r| <= tol*|r0| (mode 1), then
// beta = r.z_new / r.z.
// ---------------------------------------------------------------------------
// Last block of an update: fixed-order reduction of the block partials and
// the per-column stop test / beta (shared by both update kernels).
template <int KR>
__device__ __forceinline__ void update_finish(int init, ColState* __restrict__ cs, PcgGlobal* __restrict__ G,
                                              const double* __restrict__ part) {
  __shared__ int s_alldone;
  __shared__ double sfin[RED_THREADS];
  if (threadIdx.x == 0) s_alldone = 1;
  // parallel fixed-order reduction of the block partials: thread t owns
  // quantity t % (4*KR) of blocks t/(4*KR), t/(4*KR) + RED_THREADS/(4*KR), ...
  {
    constexpr int NQ = 4 * KR;
    const int q = threadIdx.x % 4;
    double v = 0.0;
    for (int idx = threadIdx.x; idx < (int)gridDim.x * NQ; idx += RED_THREADS) {
      double x = __ldcg(part + idx);
      v = (q < 2) ? fmax(v, x) : v + x;
    }
    sfin[threadIdx.x] = v;
  }
  __syncthreads();
  const int it = init ? 0 : G->it + 1;
  if (threadIdx.x < KR) {
    const int jj = threadIdx.x;
    constexpr int NQ = 4 * KR;
    ColState& c = cs[jj];
    double a = 0.0, b = 0.0, s = 0.0, q = 0.0;
    for (int t = jj * 4; t < RED_THREADS; t += NQ) {
      a = fmax(a, sfin[t]); b = fmax(b, sfin[t + 1]); s += sfin[t + 2]; q += sfin[t + 3];
    }
    if (init) {
      if (c.active) {
        // keep_dir (G->mode & 2): continue the previous search direction after a
        // residual replacement, beta = r.z_new / r.z of the last completed step
        c.beta = (G->mode & 2) ? s / c.rz : 0.0;
        c.alpha = 0.0;   // the fused step's first vector update is empty
        c.rz = s; c.rr0 = q; c.rr = q; c.done = 0; c.failed = 0; c.iters = 0;
      } else {
        c.done = 1;
      }
    } else if (c.active && !c.done) {
      c.maxp = a; c.maxu = b; c.rr = q;
      bool stop = ((G->mode & 1) == 0) ? (fabs(c.alpha) * a / b <= c.tol) : (q <= c.tol * c.tol * c.rr0);
      if (stop) {
        c.done = 1; c.iters = it;
      } else if (it >= G->maxiter) {
        c.done = 1; c.failed = 1; c.iters = G->maxiter + 1;
      } else {
        c.beta = s / c.rz;
        c.rz = s;
      }
    }
    if (jj < G->kcols && c.active && !c.done) atomicAnd(&s_alldone, 0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    G->it = it;
    G->all_done = s_alldone;
    G->cntC = 0;
  }
}
template <typename V, int KR>
__global__ void __launch_bounds__(RED_THREADS) k_pcg_update(
    int n1, V* __restrict__ u, V* __restrict__ r, V* __restrict__ z, const V* __restrict__ p,
    const V* __restrict__ kp, const V* __restrict__ f, const V* __restrict__ dprecon, int init,
    ColState* __restrict__ cs, PcgGlobal* __restrict__ G, double* __restrict__ part) {
  if (G->all_done) return;
  const int j = threadIdx.x & (KR - 1);
  const bool live = cs[j].active && (init || !cs[j].done);
  const V alpha = (V)(init ? 0.0 : cs[j].alpha);
  V mpv = (V)0, muv = (V)0;
  DotAcc<V> rza, rra;
  if (live) {
    const size_t n = (size_t)n1 * KR;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (init) {
      for (; i < n; i += stride) {
        V ri = f[i] - kp[i];
        V zi = dprecon[i / KR] * ri;
        r[i] = ri;
        z[i] = zi;
        rza.add(ri, zi);
        rra.add(ri, ri);
      }
    } else {
      // four independent rows per trip keep enough loads in flight
      constexpr int U = 4;
      for (; i + (U - 1) * stride < n; i += U * stride) {
        V pi[U], ui[U], ri[U], ki[U], di[U];
#pragma unroll
        for (int q = 0; q < U; ++q) {
          const size_t o = i + q * stride;
          pi[q] = p[o]; ui[q] = u[o]; ri[q] = r[o]; ki[q] = kp[o]; di[q] = dprecon[o / KR];
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
          const size_t o = i + q * stride;
          V un = fmav<V>(alpha, pi[q], ui[q]);
          V rn = fmav<V>(-alpha, ki[q], ri[q]);
          V zn = di[q] * rn;
          u[o] = un; r[o] = rn; z[o] = zn;
          mpv = fmax(mpv, fabs(pi[q]));
          muv = fmax(muv, fabs(un));
          rza.add(rn, zn);
          rra.add(rn, rn);
        }
      }
      for (; i < n; i += stride) {
        V pi = p[i];
        V un = fmav<V>(alpha, pi, u[i]);
        V rn = fmav<V>(-alpha, kp[i], r[i]);
        V zn = dprecon[i / KR] * rn;
        u[i] = un; r[i] = rn; z[i] = zn;
        mpv = fmax(mpv, fabs(pi));
        muv = fmax(muv, fabs(un));
        rza.add(rn, zn);
        rra.add(rn, rn);
      }
    }
  }
  double mp = (double)mpv, mu = (double)muv, rz = rza.value(), rr = rra.value();
  __shared__ double sred[RED_THREADS / 32][KR][4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  mp = warp_col_reduce<KR>(mp, 1);
  mu = warp_col_reduce<KR>(mu, 1);
  rz = warp_col_reduce<KR>(rz, 0);
  rr = warp_col_reduce<KR>(rr, 0);
  if (lane < KR) {
    sred[warp][lane][0] = mp; sred[warp][lane][1] = mu; sred[warp][lane][2] = rz; sred[warp][lane][3] = rr;
  }
  __syncthreads();
  if (threadIdx.x < KR) {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) {
      a = fmax(a, sred[w][threadIdx.x][0]); b = fmax(b, sred[w][threadIdx.x][1]);
      c += sred[w][threadIdx.x][2]; d += sred[w][threadIdx.x][3];
    }
    double* o = part + ((size_t)blockIdx.x * KR + threadIdx.x) * 4;
    o[0] = a; o[1] = b; o[2] = c; o[3] = d;
  }
  if (!last_block(&G->cntC)) return;
  update_finish<KR>(init, cs, G, part);
}

// FP32 update with KR = 4, 8 or 16 in 16-byte pieces: thread t always owns
// columns c0..c0+3 (c0 = 4 (t mod KR/4)) of the rows it visits, so every load
// moves 16 bytes; per-column max-norms and compensated dots are then reduced
// over the lanes of equal c0 and finished exactly as in k_pcg_update.
template <int KR>
__global__ void __launch_bounds__(RED_THREADS, 4) k_pcg_update4(
    int n1, float* __restrict__ u, float* __restrict__ r, float* __restrict__ z, const float* __restrict__ p,
    const float* __restrict__ kp, const float* __restrict__ f, const float* __restrict__ dprecon, int init,
    ColState* __restrict__ cs, PcgGlobal* __restrict__ G, double* __restrict__ part) {
  if (G->all_done) return;
  constexpr int QP = KR / 4;
  const int c0 = 4 * (threadIdx.x % QP);
  bool live[4];
  float alpha[4];
  bool any = false;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    live[k] = cs[c0 + k].active && (init || !cs[c0 + k].done);
    alpha[k] = (float)(init ? 0.0 : cs[c0 + k].alpha);
    any = any || live[k];
  }
  const bool all4 = live[0] && live[1] && live[2] && live[3];
  float mpv[4] = {0.f, 0.f, 0.f, 0.f}, muv[4] = {0.f, 0.f, 0.f, 0.f};
  DotAcc<float> rza[4], rra[4];
  if (any) {
    const size_t n4 = (size_t)n1 * QP;                    // 16-byte pieces
    const size_t stride = (size_t)gridDim.x * blockDim.x;  // a multiple of QP: c0 is fixed
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float4* p4 = reinterpret_cast<const float4*>(p);
    const float4* k4 = reinterpret_cast<const float4*>(kp);
    float4* u4 = reinterpret_cast<float4*>(u);
    float4* r4 = reinterpret_cast<float4*>(r);
    float4* z4 = reinterpret_cast<float4*>(z);
    if (init) {
      const float4* f4 = reinterpret_cast<const float4*>(f);
      for (; i < n4; i += stride) {
        const float4 fv = f4[i], kv = k4[i];
        const float d = dprecon[i / QP];
        float4 rn, zn;
        rn.x = fv.x - kv.x; rn.y = fv.y - kv.y; rn.z = fv.z - kv.z; rn.w = fv.w - kv.w;
        zn.x = d * rn.x; zn.y = d * rn.y; zn.z = d * rn.z; zn.w = d * rn.w;
        const float rv[4] = {rn.x, rn.y, rn.z, rn.w}, zv[4] = {zn.x, zn.y, zn.z, zn.w};
        if (all4) {
          r4[i] = rn;
          z4[i] = zn;
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (live[k]) { r[4 * i + k] = rv[k]; z[4 * i + k] = zv[k]; }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (live[k]) { rza[k].add(rv[k], zv[k]); rra[k].add(rv[k], rv[k]); }
      }
    } else {
      // four 16-byte loads per thread in flight, four CTAs per SM
      constexpr int U = 1;
      for (; i < n4; i += U * stride) {
        float4 pv[U], uv[U], rv[U], kv[U];
        float dv[U];
        bool in[U];
#pragma unroll
        for (int q = 0; q < U; ++q) {
          const size_t o = i + q * stride;
          in[q] = o < n4;
          if (in[q]) { pv[q] = p4[o]; uv[q] = u4[o]; rv[q] = r4[o]; kv[q] = k4[o]; dv[q] = dprecon[o / QP]; }
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
          if (!in[q]) continue;
          const size_t o = i + q * stride;
          const float pa[4] = {pv[q].x, pv[q].y, pv[q].z, pv[q].w};
          const float ua[4] = {uv[q].x, uv[q].y, uv[q].z, uv[q].w};
          const float ra[4] = {rv[q].x, rv[q].y, rv[q].z, rv[q].w};
          const float ka[4] = {kv[q].x, kv[q].y, kv[q].z, kv[q].w};
          float un[4], rn[4], zn[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            un[k] = fmaf(alpha[k], pa[k], ua[k]);
            rn[k] = fmaf(-alpha[k], ka[k], ra[k]);
            zn[k] = dv[q] * rn[k];
            if (live[k]) {
              mpv[k] = fmaxf(mpv[k], fabsf(pa[k]));
              muv[k] = fmaxf(muv[k], fabsf(un[k]));
              rza[k].add(rn[k], zn[k]);
              rra[k].add(rn[k], rn[k]);
            }
          }
          if (all4) {
            u4[o] = make_float4(un[0], un[1], un[2], un[3]);
            r4[o] = make_float4(rn[0], rn[1], rn[2], rn[3]);
            z4[o] = make_float4(zn[0], zn[1], zn[2], zn[3]);
          } else {
            // columns that are not live are left untouched
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (live[k]) { u[4 * o + k] = un[k]; r[4 * o + k] = rn[k]; z[4 * o + k] = zn[k]; }
          }
        }
      }
    }
  }
  __shared__ double sred[RED_THREADS / 32][KR][4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double mp = (double)mpv[k], mu = (double)muv[k], rz = live[k] ? rza[k].value() : 0.0,
           rr = live[k] ? rra[k].value() : 0.0;
#pragma unroll
    for (int o = 16; o >= QP; o >>= 1) {
      mp = fmax(mp, __shfl_xor_sync(FULL, mp, o));
      mu = fmax(mu, __shfl_xor_sync(FULL, mu, o));
      rz += __shfl_xor_sync(FULL, rz, o);
      rr += __shfl_xor_sync(FULL, rr, o);
    }
    if (lane < QP) {
      const int j = 4 * lane + k;
      sred[warp][j][0] = mp; sred[warp][j][1] = mu; sred[warp][j][2] = rz; sred[warp][j][3] = rr;
    }
  }
  __syncthreads();
  if (threadIdx.x < KR) {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int w = 0; w < RED_THREADS / 32; ++w) {
      a = fmax(a, sred[w][threadIdx.x][0]); b = fmax(b, sred[w][threadIdx.x][1]);
      c += sred[w][threadIdx.x][2]; d += sred[w][threadIdx.x][3];
    }
    double* o = part + ((size_t)blockIdx.x * KR + threadIdx.x) * 4;
    o[0] = a; o[1] = b; o[2] = c; o[3] = d;
  }
  if (!last_block(&G->cntC)) return;
  update_finish<KR>(init, cs, G, part);
}

template <typename V, int KR>
void pcg_update(int n1, V* u, V* r, V* z, const V* p, const V* kp, const V* f, const V* dprecon, int init,
                ColState* cs, PcgGlobal* G, double* part, cudaStream_t s) {
  if constexpr (std::is_same<V, float>::value && (KR == 4 || KR == 8 || KR == 16)) {
    SG_LAUNCH k_pcg_update4<KR><<<red_grid((size_t)n1 * (KR / 4), RED_THREADS * 4, NPART), RED_THREADS, 0, s>>>(
        n1, u, r, z, p, kp, f, dprecon, init, cs, G, part);
    return;
  }
  SG_LAUNCH k_pcg_update<V, KR><<<red_grid((size_t)n1 * KR, RED_THREADS * 4, NPART), RED_THREADS, 0, s>>>(
      n1, u, r, z, p, kp, f, dprecon, init, cs, G, part);
}

// ---------------------------------------------------------------------------
// K5: one stress / yield / flow / body-load pass for one trial.
// One warp per element, lane i < 27 = GLL point i.  Mirrors src/slope.F90:311-383:
// eps = B x_e - evpt; sigma = C eps; eff = sigma + stress; invariants
// (stress_invariant), F (mohcouf); if F >= 0: dQ (mohcouq), M1..M3 (formm),
// flow = F (M1 dq1 + M2 dq2 + M3 dq3), evp = flow eff dt, evpt += evp and,
// unless finalising, bload += B^T (C evp) detJ w; when finalising, stress = eff.
// Yb receives the element body-load vector (zeros when finalising), to be
// gathered in element order into bodyload.
// ---------------------------------------------------------------------------
constexpr int STRESS_WARPS = 4;
constexpr double DEG2RAD_D = 3.141592653589793 / 180.0;

__device__ __forceinline__ void stress_invariant_d(const double* s, double& sigm, double& dsbar, double& theta) {
  const double small = 1.e-12, three = 3.0, six = 6.0;
  const double sq3 = sqrt(three);
  double s1 = s[0], s2 = s[1], s3 = s[2], s4 = s[3], s5 = s[4], s6 = s[5];
  sigm = (s1 + s2 + s3) / three;
  double d2 = ((s1 - s2) * (s1 - s2) + (s2 - s3) * (s2 - s3) + (s3 - s1) * (s3 - s1)) / six + s4 * s4 + s5 * s5 +
              s6 * s6;
  if (d2 < small) d2 = small;
  double ds1 = s1 - sigm, ds2 = s2 - sigm, ds3 = s3 - sigm;
  double d3 = ds1 * ds2 * ds3 - ds1 * s5 * s5 - ds2 * s6 * s6 - ds3 * s4 * s4 + 2.0 * s4 * s5 * s6;
  double sq = sqrt(d2);
  dsbar = sq3 * sq;
  if (dsbar < small) {
    theta = 0.0;
  } else {
    double sine = -three * sq3 * d3 / (2.0 * (sq * sq * sq));
    if (sine >= 1.0) sine = 1.0;
    if (sine < -1.0) sine = -1.0;
    theta = asin(sine) / three;
  }
}

__global__ void __launch_bounds__(STRESS_WARPS * 32) k_stress_update(
    const double* __restrict__ geo, const int* __restrict__ elist, int nel, const int* __restrict__ ge,
    const int* __restrict__ mat_id, const double* __restrict__ x, int xstride, int xcol, const MatF* __restrict__ mf,
    double dt, int nl_isconv, int finalize, double* __restrict__ evpt, double* __restrict__ stress,
    double* __restrict__ Yb, int ystride, int ycol, double* __restrict__ fmax_part, const int* __restrict__ pos,
    double* __restrict__ vm_pt, double* __restrict__ sf_pt, const double* __restrict__ wp,
    const int* __restrict__ gnum, int wp_first) {
  __shared__ double s_eld[STRESS_WARPS][NEDOF];
  __shared__ double s_q[STRESS_WARPS][NGLL][9];
  __shared__ double s_fmax[STRESS_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool want_bload = !nl_isconv && !finalize;
  double fmax_l = 0.0;
  for (int le = blockIdx.x * STRESS_WARPS + warp; le < nel; le += gridDim.x * STRESS_WARPS) {
    const int e = elist ? elist[le] : le;
    const MatF m = mf[mat_id[e] - 1];
    for (int t = lane; t < NEDOF; t += 32) s_eld[warp][t] = x[(size_t)ge[(size_t)e * NEDOF + t] * xstride + xcol];
    __syncwarp();
    if (lane < NGLL) {
      const int i = lane;
      const int ic[3] = {i % 3, (i / 3) % 3, i / 9};
      const double* gp = geo + ((size_t)e * NGLL + i) * GEO_STRIDE;
      double Ji[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) Ji[t] = gp[t];
      const double detj = gp[9];
      // du_c/dxi_a from the three nodes on the line through i along a
      double dU[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        int stride = (a == 0) ? 1 : (a == 1 ? 3 : 9);
        int base = i - ic[a] * stride;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double s = 0.0;
#pragma unroll
          for (int mm = 0; mm < 3; ++mm) s = s + c_D[ic[a]][mm] * s_eld[warp][3 * (base + mm * stride) + c];
          dU[c][a] = s;
        }
      }
      // G[c][d] = du_c/dx_d = sum_a Jinv(d,a) dU[c][a]
      double Gm[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) Gm[c][d] = Ji[3 * d] * dU[c][0] + Ji[3 * d + 1] * dU[c][1] + Ji[3 * d + 2] * dU[c][2];
      double* ev = evpt + ((size_t)e * NGLL + i) * NST;
      double* se = stress + ((size_t)e * NGLL + i) * NST;
      double eps[6] = {Gm[0][0], Gm[1][1], Gm[2][2], Gm[0][1] + Gm[1][0], Gm[1][2] + Gm[2][1], Gm[2][0] + Gm[0][2]};
      double evl[6];
#pragma unroll
      for (int s = 0; s < 6; ++s) { evl[s] = ev[s]; eps[s] = eps[s] - evl[s]; }
      double sig[6];
      sig[0] = m.c11 * eps[0] + m.c12 * eps[1] + m.c12 * eps[2];
      sig[1] = m.c12 * eps[0] + m.c11 * eps[1] + m.c12 * eps[2];
      sig[2] = m.c12 * eps[0] + m.c12 * eps[1] + m.c11 * eps[2];
      sig[3] = m.c44 * eps[3]; sig[4] = m.c44 * eps[4]; sig[5] = m.c44 * eps[5];
      // effective stress; the pore pressure p of the point's node (0 off the
      // submerged nodes) is added to the normal components, after the stored
      // stress in the slope form (src/slope.F90:334-341) and before it in the
      // excavation form (src/excavation.F90:566-576)
      double eff[6];
      if (wp) {
        const double pw = wp[gnum[(size_t)e * NGLL + i]];
#pragma unroll
        for (int s = 0; s < 6; ++s) {
          if (s >= 3) eff[s] = sig[s] + se[s];
          else if (wp_first) eff[s] = (sig[s] + pw) + se[s];
          else eff[s] = (sig[s] + se[s]) + pw;
        }
      } else {
#pragma unroll
        for (int s = 0; s < 6; ++s) eff[s] = sig[s] + se[s];
      }
      double sigm, dsbar, theta;
      stress_invariant_d(eff, sigm, dsbar, theta);
      double snth, csth;
      sincos(theta, &snth, &csth);
      const double r3 = 3.0, sq3 = sqrt(3.0);
      // mohcouf (src/plastic_library.f90:95-108)
      double f = m.snph * sigm + dsbar * (csth / sq3 - snth * m.snph / r3) - m.cohf * m.csph;
      fmax_l = fmax(fmax_l, f);
      double q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      if (f >= 0.0) {
        // mohcouq (src/plastic_library.f90:116-143)
        double dq1 = m.snps, dq2, dq3;
        if (fabs(snth) > 0.49) {
          double c1 = snth < 0.0 ? -1.0 : 1.0;
          dq2 = (sq3 * 0.5 - c1 * m.snps * 0.5 / sq3) * sq3 * 0.5 / dsbar;
          dq3 = 0.0;
        } else {
          double cs3th = cos(r3 * theta), tn3th = tan(r3 * theta), tnth = snth / csth;
          dq2 = sq3 * csth / dsbar * ((1.0 + tnth * tn3th) + m.snps * (tn3th - tnth) / sq3) * 0.5;
          dq3 = 0.5 * r3 * (sq3 * snth + m.snps * csth) / (cs3th * dsbar * dsbar);
        }
        // formm (src/plastic_library.f90:150-208): M1, M2, M3 (divided by 3)
        const double sx = eff[0], sy = eff[1], sz = eff[2], txy = eff[3], tyz = eff[4], tzx = eff[5];
        const double sgm = (sx + sy + sz) / r3;
        const double dx = sx - sgm, dy = sy - sgm, dz = sz - sgm;
        double M[6][6];
        const double m1v = 1.0 / (r3 * sgm) / r3;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
          for (int b = 0; b < 6; ++b) M[a][b] = 0.0;
        double m3[6][6];
        m3[0][0] = dx; m3[0][1] = dz; m3[0][2] = dy; m3[0][3] = txy; m3[0][4] = -2.0 * tyz; m3[0][5] = tzx;
        m3[1][1] = dy; m3[1][2] = dx; m3[1][3] = txy; m3[1][4] = tyz; m3[1][5] = -2.0 * tzx;
        m3[2][2] = dz; m3[2][3] = -2.0 * txy; m3[2][4] = tyz; m3[2][5] = tzx;
        m3[3][3] = -r3 * dz; m3[3][4] = r3 * tzx; m3[3][5] = r3 * tyz;
        m3[4][4] = -r3 * dx; m3[4][5] = r3 * txy;
        m3[5][5] = -r3 * dy;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
          for (int b = a; b < 6; ++b) {
            double m1 = (a < 3 && b < 3) ? m1v : 0.0;
            double m2 = 0.0;
            if (a == b) m2 = (a < 3 ? 2.0 : 6.0) / r3;
            else if (b < 3) m2 = -1.0 / r3;
            double v = f * (m1 * dq1 + m2 * dq2 + (m3[a][b] / r3) * dq3);
            M[a][b] = v;
            M[b][a] = v;
          }
        double evp[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) {
          double s = 0.0;
#pragma unroll
          for (int b = 0; b < 6; ++b) s = s + M[a][b] * eff[b];
          evp[a] = s * dt;
          ev[a] = evl[a] + evp[a];
        }
        if (want_bload) {
          double dv[6];
          dv[0] = m.c11 * evp[0] + m.c12 * evp[1] + m.c12 * evp[2];
          dv[1] = m.c12 * evp[0] + m.c11 * evp[1] + m.c12 * evp[2];
          dv[2] = m.c12 * evp[0] + m.c12 * evp[1] + m.c11 * evp[2];
          dv[3] = m.c44 * evp[3]; dv[4] = m.c44 * evp[4]; dv[5] = m.c44 * evp[5];
          const double S[3][3] = {{dv[0], dv[3], dv[5]}, {dv[3], dv[1], dv[4]}, {dv[5], dv[4], dv[2]}};
          const double wd = detj * c_w[i];
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int a = 0; a < 3; ++a)
              q[3 * c + a] = (S[c][0] * Ji[a] + S[c][1] * Ji[3 + a] + S[c][2] * Ji[6 + a]) * wd;
        }
      }
      if (finalize) {
#pragma unroll
        for (int s = 0; s < 6; ++s) se[s] = eff[s];
        // excavation fields (src/excavation.F90:599-609): von Mises effective
        // plastic strain of the updated evpt and the point's safety factor
        if (vm_pt) {
          double q2 = 0.0;
#pragma unroll
          for (int s = 0; s < 6; ++s) q2 = q2 + ev[s] * ev[s];
          vm_pt[(size_t)le * NGLL + i] = sqrt((2.0 / r3) * q2);
        }
        if (sf_pt)
          sf_pt[(size_t)le * NGLL + i] =
              (sigm * m.snph - m.cohf * m.csph) / (-dsbar * (csth / sq3 - snth * m.snph / r3));
      }
#pragma unroll
      for (int t = 0; t < 9; ++t) s_q[warp][i][t] = q[t];
    }
    __syncwarp();
    if (Yb && lane < NGLL) {
      // node n = lane: F_n[c] = sum over points i on the lines through n, in
      // increasing i, of sum_a Q_i[c][a] * dlagrange(a,i,n)
      const int n = lane;
      const int nc[3] = {n % 3, (n / 3) % 3, n / 9};
      double F[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < NGLL; ++i) {
        const int ic[3] = {i % 3, (i / 3) % 3, i / 9};
        int ndiff = (ic[0] != nc[0]) + (ic[1] != nc[1]) + (ic[2] != nc[2]);
        if (ndiff > 1) continue;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          bool ok = true;
#pragma unroll
          for (int b = 0; b < 3; ++b)
            if (b != a && ic[b] != nc[b]) ok = false;
          if (!ok) continue;
          double dl = c_D[ic[a]][nc[a]];
#pragma unroll
          for (int c = 0; c < 3; ++c) F[c] = F[c] + s_q[warp][i][3 * c + a] * dl;
        }
      }
      const int q = pos[(size_t)le * NGLL + n];
      if (q >= 0) {
        double* yo = Yb + ((size_t)q * 3) * ystride + ycol;
        yo[0] = F[0]; yo[ystride] = F[1]; yo[2 * ystride] = F[2];
      }
    }
    __syncwarp();
  }
  // fmax partial per block
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) fmax_l = fmax(fmax_l, __shfl_xor_sync(FULL, fmax_l, o));
  if (lane == 0) s_fmax[warp] = fmax_l;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < STRESS_WARPS; ++w) v = fmax(v, s_fmax[w]);
    fmax_part[blockIdx.x] = v;
  }
}

void launch_stress_update(const double* geo, const int* elist, int nel, const int* ge_glob, const int* mat_id,
                          const double* x, int xstride, int xcol, const MatF* mf, double dt, int nl_isconv,
                          int finalize, double* evpt, double* stress, double* Yb, int ystride, int ycol,
                          double* fmax_part, const int* pos, cudaStream_t s, double* vm_pt, double* sf_pt,
                          const double* wp, const int* gnum, int wp_first) {
  // fixed grid so that fmax_part has NPART entries
  SG_LAUNCH k_stress_update<<<NPART, STRESS_WARPS * 32, 0, s>>>(geo, elist, nel, ge_glob, mat_id, x, xstride, xcol, mf, dt,
                                                       nl_isconv, finalize, evpt, stress, Yb, ystride, ycol,
                                                       fmax_part, pos, vm_pt, sf_pt, wp, gnum, wp_first);
}

// ---------------------------------------------------------------------------
// compute_pressure (src/compute_pressure.f90:10-186): hydrostatic pressure
// gamw (z - z_node) under a water table, on the nodes of the elements whose
// material is a water material.  k_mark_submerged flags those nodes;
// k_water_pressure gives each node one thread that scans the surfaces in file
// order and stops at the first one the node lies under (the reference's
// `cycle nodal`).  Surface kinds: 0 horizontal line z1 over rdir in [rx1, rx2];
// 1 inclined line z1 -> z2 over rdir in [min(rx1,rx2), max(rx1,rx2)];
// 2 meshed faces, with the reference's plane offset D = det[xf1 xf2 xf3] taken
// as it is written (z = -(A x + B y + D)/C), a vertical face taking its top z,
// and a z outside the face's z range stopping the computation with an error
// (err, INT_MAX on entry, receives the smallest failing node + 1); nvert counts
// vertical faces met.
// ---------------------------------------------------------------------------
__global__ void k_mark_submerged(const int* __restrict__ g_num, const int* __restrict__ mat_id,
                                 const int* __restrict__ water_mat, int nelmt, int* __restrict__ sub) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelmt * NGLL) return;
  if (water_mat[mat_id[t / NGLL] - 1]) sub[g_num[t]] = 1;
}

// corner nodes (0-based GLL numbering) of Exodus faces 1..6, the reference's
// hexface(:)%gnode for NGLL = 3 (src/element.f90:107-124)
__constant__ int c_face_corner[6][4] = {{0, 2, 20, 18}, {2, 8, 26, 20}, {6, 8, 26, 24},
                                        {0, 6, 24, 18}, {0, 2, 8, 6},   {18, 20, 26, 24}};

__global__ void k_water_pressure(int nnode, const double* __restrict__ g_coord, const int* __restrict__ sub,
                                 const WaterSurface* __restrict__ surf, int nsurf, const int* __restrict__ face,
                                 const int* __restrict__ g_num, double* __restrict__ wp, int* __restrict__ err,
                                 int* __restrict__ nvert) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnode) return;
  const double gamw = 9.81;
  double p = 0.0;
  if (sub[n]) {
    const double xp[3] = {g_coord[3 * (size_t)n], g_coord[3 * (size_t)n + 1], g_coord[3 * (size_t)n + 2]};
    bool done = false;
    for (int w = 0; w < nsurf && !done; ++w) {
      const WaterSurface S = surf[w];
      if (S.stype == 0) {
        const double r = xp[S.rdir - 1], z = S.z1;
        if (r >= S.rx1 && r <= S.rx2 && xp[2] <= z) {
          if (z > xp[2]) p = gamw * (z - xp[2]);
          done = true;
        }
      } else if (S.stype == 1) {
        const double r = xp[S.rdir - 1];
        if (r >= fmin(S.rx1, S.rx2) && r <= fmax(S.rx1, S.rx2) && xp[2] <= fmax(S.z1, S.z2)) {
          const double z = S.z1 + (S.z2 - S.z1) * (r - S.rx1) / (S.rx2 - S.rx1);
          if (z > xp[2]) p = gamw * (z - xp[2]);
          done = true;
        }
      } else {
        for (int f = 0; f < S.nface && !done; ++f) {
          const int e = face[2 * (S.face0 + f)], fc = face[2 * (S.face0 + f) + 1];
          double xf[3][4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int nd = g_num[(size_t)e * NGLL + c_face_corner[fc - 1][k]];
#pragma unroll
            for (int c = 0; c < 3; ++c) xf[c][k] = g_coord[3 * (size_t)nd + c];
          }
          double lo[3], hi[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lo[c] = fmin(fmin(xf[c][0], xf[c][1]), fmin(xf[c][2], xf[c][3]));
            hi[c] = fmax(fmax(xf[c][0], xf[c][1]), fmax(xf[c][2], xf[c][3]));
          }
          if (!(xp[0] >= lo[0] && xp[0] <= hi[0] && xp[1] >= lo[1] && xp[1] <= hi[1] && xp[2] <= hi[2])) continue;
          const double v1[3] = {xf[0][1] - xf[0][0], xf[1][1] - xf[1][0], xf[2][1] - xf[2][0]};
          const double v2[3] = {xf[0][2] - xf[0][0], xf[1][2] - xf[1][0], xf[2][2] - xf[2][0]};
          const double A = v1[1] * v2[2] - v2[1] * v1[2];
          const double B = v2[0] * v1[2] - v1[0] * v2[2];
          const double C = v1[0] * v2[1] - v2[0] * v1[1];
          // determinant of the 3x3 matrix whose columns are the first three corners
          const double D = xf[0][0] * (xf[1][1] * xf[2][2] - xf[2][1] * xf[1][2]) -
                           xf[0][1] * (xf[1][0] * xf[2][2] - xf[2][0] * xf[1][2]) +
                           xf[0][2] * (xf[1][0] * xf[2][1] - xf[2][0] * xf[1][1]);
          double z;
          if (C == 0.0) {
            atomicAdd(nvert, 1);
            z = hi[2];
          } else {
            z = -(A * xp[0] + B * xp[1] + D) / C;
          }
          if (z > hi[2] || z < lo[2]) {
            atomicMin(err, n + 1);
            return;
          }
          if (z > xp[2]) p = gamw * (z - xp[2]);
          done = true;
        }
      }
    }
  }
  wp[n] = p;
}

void launch_water_pressure(int nnode, int nelmt, const double* g_coord, const int* g_num, const int* mat_id,
                           const int* water_mat, const WaterSurface* surf, int nsurf, const int* face, int* sub,
                           double* wp, int* err, int* nvert, cudaStream_t s) {
  cudaMemsetAsync(sub, 0, sizeof(int) * (size_t)nnode, s);
  if (nelmt > 0)
    SG_LAUNCH k_mark_submerged<<<(nelmt * NGLL + 255) / 256, 256, 0, s>>>(g_num, mat_id, water_mat, nelmt, sub);
  if (nnode > 0)
    SG_LAUNCH k_water_pressure<<<(nnode + 255) / 256, 256, 0, s>>>(nnode, g_coord, sub, surf, nsurf, face, g_num,
                                                                  wp, err, nvert);
}

// elastic_stress (src/postprocess.f90:40-79): sigma = C B x per GLL point
// (accumulate = 1 adds to the existing stress, the elastic_stress_intact form).
__global__ void k_elastic_stress(const double* __restrict__ geo, const int* __restrict__ elist, int nel,
                                 const int* __restrict__ ge, const int* __restrict__ mat_id,
                                 const double* __restrict__ x, int xstride, int xcol, const MatF* __restrict__ mf,
                                 int accumulate, double* __restrict__ stress) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nel * NGLL) return;
  int le = t / NGLL, i = t - le * NGLL;
  int e = elist ? elist[le] : le;
  const MatF m = mf[mat_id[e] - 1];
  const int ic[3] = {i % 3, (i / 3) % 3, i / 9};
  const double* gp = geo + ((size_t)e * NGLL + i) * GEO_STRIDE;
  const int* g = ge + (size_t)e * NEDOF;
  double dU[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int stride = (a == 0) ? 1 : (a == 1 ? 3 : 9);
    int base = i - ic[a] * stride;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double s = 0.0;
#pragma unroll
      for (int mm = 0; mm < 3; ++mm) s = s + c_D[ic[a]][mm] * x[(size_t)g[3 * (base + mm * stride) + c] * xstride + xcol];
      dU[c][a] = s;
    }
  }
  double Gm[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 0; d < 3; ++d) Gm[c][d] = gp[3 * d] * dU[c][0] + gp[3 * d + 1] * dU[c][1] + gp[3 * d + 2] * dU[c][2];
  double eps[6] = {Gm[0][0], Gm[1][1], Gm[2][2], Gm[0][1] + Gm[1][0], Gm[1][2] + Gm[2][1], Gm[2][0] + Gm[0][2]};
  double sig[6];
  sig[0] = m.c11 * eps[0] + m.c12 * eps[1] + m.c12 * eps[2];
  sig[1] = m.c12 * eps[0] + m.c11 * eps[1] + m.c12 * eps[2];
  sig[2] = m.c12 * eps[0] + m.c12 * eps[1] + m.c11 * eps[2];
  sig[3] = m.c44 * eps[3]; sig[4] = m.c44 * eps[4]; sig[5] = m.c44 * eps[5];
  double* se = stress + ((size_t)e * NGLL + i) * NST;
#pragma unroll
  for (int s = 0; s < 6; ++s) se[s] = accumulate ? se[s] + sig[s] : sig[s];
}

void launch_elastic_stress(const double* geo, const int* elist, int nel, const int* ge_glob, const int* mat_id,
                           const double* x, int xstride, int xcol, const MatF* mf, int accumulate, double* stress,
                           cudaStream_t s) {
  int n = nel * NGLL;
  if (n > 0) SG_LAUNCH k_elastic_stress<<<(n + 127) / 128, 128, 0, s>>>(geo, elist, nel, ge_glob, mat_id, x, xstride, xcol, mf,
                                                              accumulate, stress);
}

// overburden_stress (src/postprocess.f90:10-33)
__global__ void k_overburden(const double* __restrict__ g_coord, const int* __restrict__ g_num,
                             const int* __restrict__ mat_id, const double* __restrict__ gam, int nelmt, double z0,
                             double p0, double k0, double* __restrict__ stress) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelmt * NGLL) return;
  int e = t / NGLL;
  double z = g_coord[(size_t)3 * g_num[t] + 2];
  double szz = p0 - gam[mat_id[e] - 1] * fabs(z - z0);
  double* s = stress + (size_t)t * NST;
  s[2] = szz; s[0] = k0 * szz; s[1] = k0 * szz;
}

void launch_overburden(const double* g_coord, const int* g_num, const int* mat_id, const double* gam, int nelmt,
                       double z0, double p0, double k0, double* stress, cudaStream_t s) {
  int n = nelmt * NGLL;
  if (n > 0) SG_LAUNCH k_overburden<<<(n + 255) / 256, 256, 0, s>>>(g_coord, g_num, mat_id, gam, nelmt, z0, p0, k0, stress);
}

// K9: equivalent nodal load of removed elements, sum_i B_i^T sigma_i detJ w
// plus gamma detJ w on the z dof of node i (excavation_load_nodal,
// src/excavation_library.f90:186-236).  One thread per (element, node).
__global__ void k_release_load(const double* __restrict__ geo, const int* __restrict__ elist, int nel,
                               const int* __restrict__ mat_id, const double* __restrict__ gam,
                               const double* __restrict__ stress, double* __restrict__ Ye,
                               const int* __restrict__ pos) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nel * NGLL) return;
  int le = t / NGLL, n = t - le * NGLL;
  int e = elist[le];
  double F[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < NGLL; ++i) {
    if (!on_line(i, n)) continue;
    const double* gp = geo + ((size_t)e * NGLL + i) * GEO_STRIDE;
    double g[3];
    point_grad(gp, i, n, g);
    const double* sg = stress + ((size_t)e * NGLL + i) * NST;
    double wd = gp[9] * c_w[i];
    F[0] = F[0] + (sg[0] * g[0] + sg[3] * g[1] + sg[5] * g[2]) * wd;
    F[1] = F[1] + (sg[1] * g[1] + sg[3] * g[0] + sg[4] * g[2]) * wd;
    F[2] = F[2] + (sg[2] * g[2] + sg[4] * g[1] + sg[5] * g[0]) * wd;
  }
  const double* gn = geo + ((size_t)e * NGLL + n) * GEO_STRIDE;
  double eld = gn[9] * c_w[n];
  const int q = pos[(size_t)le * NGLL + n];
  if (q < 0) return;
  double* yo = Ye + (size_t)q * 3;
  yo[0] = F[0];
  yo[1] = F[1];
  yo[2] = eld * gam[mat_id[e] - 1] + F[2];
}

void launch_release_load(const double* geo, const int* elist, int nel, const int* mat_id, const double* gam,
                         const double* stress, double* Ye, const int* pos, cudaStream_t s) {
  int n = nel * NGLL;
  if (n > 0) SG_LAUNCH k_release_load<<<(n + 127) / 128, 128, 0, s>>>(geo, elist, nel, mat_id, gam, stress, Ye, pos);
}

// ---------------------------------------------------------------------------
// Small vector kernels with per-column reductions written to part[NPART][KR][q].
// ---------------------------------------------------------------------------
// K8 nl check (src/slope.F90:307-309): max|x-oldx|, max|x| per column, oldx = x.
__global__ void k_nl_check(int n1, int KR, const double* __restrict__ x, double* __restrict__ oldx,
                           double* __restrict__ part) {
  __shared__ double s[RED_THREADS][2];
  double a = 0.0, b = 0.0;
  const int j = threadIdx.x % KR;
  const size_t n = (size_t)n1 * KR;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double xi = x[i];
    a = fmax(a, fabs(xi - oldx[i]));
    b = fmax(b, fabs(xi));
    oldx[i] = xi;
  }
  s[threadIdx.x][0] = a;
  s[threadIdx.x][1] = b;
  __syncthreads();
  if (threadIdx.x < KR) {
    double A = 0.0, B = 0.0;
    for (int t = threadIdx.x; t < RED_THREADS; t += KR) { A = fmax(A, s[t][0]); B = fmax(B, s[t][1]); }
    part[((size_t)blockIdx.x * KR + j) * 2] = A;
    part[((size_t)blockIdx.x * KR + j) * 2 + 1] = B;
  }
}

void launch_nl_check(int n1, int KR, int k, const double* x, double* oldx, double* part, cudaStream_t s) {
  (void)k;
  SG_LAUNCH k_nl_check<<<NPART, RED_THREADS, 0, s>>>(n1, KR, x, oldx, part);
}

// load = extload + bodyload; load(0) = 0 (src/slope.F90:288-289)
__global__ void k_load_combine(int n1, int KR, const double* __restrict__ ext, const double* __restrict__ body,
                               double* __restrict__ load) {
  size_t n = (size_t)n1 * KR;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    size_t row = i / KR;
    load[i] = row == 0 ? 0.0 : ext[row] + body[i];
  }
}

void launch_load_combine(int n1, int KR, const double* extload, const double* bodyload, double* load,
                         cudaStream_t s) {
  SG_LAUNCH k_load_combine<<<NPART, RED_THREADS, 0, s>>>(n1, KR, extload, bodyload, load);
}

// r64 = f - kp (FP64), r32 = (float) r64; partials |r|^2, |f|^2 per column.
__global__ void k_residual(int n1, int KR, const double* __restrict__ f, const double* __restrict__ kp,
                           double* __restrict__ r64, float* __restrict__ r32, double* __restrict__ part) {
  __shared__ double s[RED_THREADS][2];
  double a = 0.0, b = 0.0;
  const int j = threadIdx.x % KR;
  const size_t n = (size_t)n1 * KR;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double ri = (i < (size_t)KR) ? 0.0 : f[i] - kp[i];
    r64[i] = ri;
    r32[i] = (float)ri;
    a += ri * ri;
    b += f[i] * f[i];
  }
  s[threadIdx.x][0] = a;
  s[threadIdx.x][1] = b;
  __syncthreads();
  if (threadIdx.x < KR) {
    double A = 0.0, B = 0.0;
    for (int t = threadIdx.x; t < RED_THREADS; t += KR) { A += s[t][0]; B += s[t][1]; }
    part[((size_t)blockIdx.x * KR + j) * 2] = A;
    part[((size_t)blockIdx.x * KR + j) * 2 + 1] = B;
  }
}

void launch_residual_norms(int n1, int KR, const double* f, const double* kp, double* r64, float* r32,
                           double* part, cudaStream_t s) {
  SG_LAUNCH k_residual<<<NPART, RED_THREADS, 0, s>>>(n1, KR, f, kp, r64, r32, part);
}

// x += d for the columns in colmask; partials max|d|, max|x| per column.
__global__ void k_axpy_corr(int n1, int KR, const int* __restrict__ colmask, const float* __restrict__ d,
                            double* __restrict__ x, double* __restrict__ part) {
  __shared__ double s[RED_THREADS][2];
  double a = 0.0, b = 0.0;
  const int j = threadIdx.x % KR;
  const bool on = colmask[j] != 0;
  const size_t n = (size_t)n1 * KR;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double xi = x[i];
    if (on) {
      double di = (double)d[i];
      xi = xi + di;
      x[i] = xi;
      a = fmax(a, fabs(di));
    }
    b = fmax(b, fabs(xi));
  }
  s[threadIdx.x][0] = a;
  s[threadIdx.x][1] = b;
  __syncthreads();
  if (threadIdx.x < KR) {
    double A = 0.0, B = 0.0;
    for (int t = threadIdx.x; t < RED_THREADS; t += KR) { A = fmax(A, s[t][0]); B = fmax(B, s[t][1]); }
    part[((size_t)blockIdx.x * KR + j) * 2] = A;
    part[((size_t)blockIdx.x * KR + j) * 2 + 1] = B;
  }
}

void launch_axpy_correction(int n1, int KR, const int* colmask, const float* d, double* x, double* part,
                            cudaStream_t s) {
  SG_LAUNCH k_axpy_corr<<<NPART, RED_THREADS, 0, s>>>(n1, KR, colmask, d, x, part);
}

// dprecon(1:) = 1/dprecon(1:), dprecon(0) = 0 (src/slope.F90:199), plus an FP32 copy.
__global__ void k_invert_diag(int n1, double* __restrict__ dp, float* __restrict__ dp32) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n1) return;
  double v = (i == 0) ? 0.0 : 1.0 / dp[i];
  dp[i] = v;
  if (dp32) dp32[i] = (float)v;
}

void launch_invert_diag(int n1, double* dprecon, float* dprecon32, cudaStream_t s) {
  SG_LAUNCH k_invert_diag<<<(n1 + 255) / 256, 256, 0, s>>>(n1, dprecon, dprecon32);
}

// explicit instantiations
#define SG_INST(V, KR)                                                                                          \
  template void pcg_apply<V, KR>(int, const void*, const int*, int, const V*, const V*, int, V*, const ColState*, \
                                 const PcgGlobal*, const int*, const int*, int*, cudaStream_t);                             \
  template void pcg_gather<V, KR>(const GatherTopo&, const V*, V*, V*, const V*, int, ColState*, PcgGlobal*,    \
                                  double*, cudaStream_t);                                                       \
  template void pcg_update<V, KR>(int, V*, V*, V*, const V*, const V*, const V*, const V*, int, ColState*,      \
                                  PcgGlobal*, double*, cudaStream_t);
SG_INST(double, 1)
SG_INST(double, 2)
SG_INST(double, 4)
SG_INST(double, 8)
SG_INST(double, 16)
SG_INST(float, 1)
SG_INST(float, 2)
SG_INST(float, 4)
SG_INST(float, 8)
SG_INST(float, 16)
template void launch_gather_plain<double>(const GatherTopo&, int, const double*, double*, int, const int*,
                                          cudaStream_t);
template void launch_gather_plain<float>(const GatherTopo&, int, const float*, float*, int, const int*,
                                         cudaStream_t);

// Fixed-order reduction of block partials part[nblk][KR][nq] into out[KR][nq];
// bit q of maxmask selects max instead of sum for quantity q.
__global__ void k_final_reduce(const double* __restrict__ part, int nblk, int KR, int nq, int maxmask,
                               double* __restrict__ out) {
  // thread t owns entry t % (KR*nq) of blocks t/(KR*nq), ...; 256 threads, KR*nq <= 64 divides 256
  __shared__ double s[256];
  const int W = KR * nq;
  const int e = threadIdx.x % W, q = e % nq;
  const bool mx = (maxmask >> q) & 1;
  double v = 0.0;
  for (int idx = threadIdx.x; idx < nblk * W; idx += blockDim.x) {
    double x = part[idx];
    v = mx ? fmax(v, x) : v + x;
  }
  s[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x < W) {
    double r = 0.0;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += W) r = mx ? fmax(r, s[t]) : r + s[t];
    out[threadIdx.x] = r;
  }
}

void launch_final_reduce(const double* part, int nblk, int KR, int nq, int maxmask, double* out, cudaStream_t s) {
  SG_LAUNCH k_final_reduce<<<1, 256, 0, s>>>(part, nblk, KR, nq, maxmask, out);
}

// Nodal displacement maxima of one column (src/slope.F90:400-415):
// part[b][0] = max |u_d| over nodes and dofs, part[b][1] = max |u| (node norm).
__global__ void k_disp_max(int nnode, const int* __restrict__ gdof, const double* __restrict__ x, int KR, int col,
                           double* __restrict__ part) {
  __shared__ double s[RED_THREADS][2];
  double a = 0.0, b = 0.0;
  for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < nnode; nd += gridDim.x * blockDim.x) {
    double u[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int g = gdof[3 * nd + d];
      u[d] = g ? x[(size_t)g * KR + col] : 0.0;
      a = fmax(a, fabs(u[d]));
    }
    b = fmax(b, sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
  }
  s[threadIdx.x][0] = a;
  s[threadIdx.x][1] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    double A = 0.0, B = 0.0;
    for (int t = 0; t < RED_THREADS; ++t) { A = fmax(A, s[t][0]); B = fmax(B, s[t][1]); }
    part[2 * blockIdx.x] = A;
    part[2 * blockIdx.x + 1] = B;
  }
}

void launch_disp_max(int nnode, const int* gdof, const double* x, int KR, int col, double* part, cudaStream_t s) {
  SG_LAUNCH k_disp_max<<<NPART, RED_THREADS, 0, s>>>(nnode, gdof, x, KR, col, part);
}

// x(:,col) /= n etc.: y[i*KR+col] = a*y[i*KR+col] (all columns when col < 0)
__global__ void k_scale(size_t n, double* __restrict__ y, double a) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = y[i] / a;
}
// zero column j of three [n1][KR] vectors (a new trial in slot j)
__global__ void k_col_zero(int n1, int KR, int j, double* __restrict__ a, double* __restrict__ b,
                           double* __restrict__ c) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1; i += gridDim.x * blockDim.x) {
    size_t o = (size_t)i * KR + j;
    a[o] = 0.0; b[o] = 0.0; c[o] = 0.0;
  }
}
void launch_col_zero(int n1, int KR, int j, double* a, double* b, double* c, cudaStream_t s) {
  SG_LAUNCH k_col_zero<<<NPART, RED_THREADS, 0, s>>>(n1, KR, j, a, b, c);
}

void launch_div(size_t n, double* y, double a, cudaStream_t s) { SG_LAUNCH k_scale<<<NPART, RED_THREADS, 0, s>>>(n, y, a); }

}  // namespace sg
