// sg_apply_mf.cu -- matrix-free FP32 element apply of the mixed form.
//
// With GLL quadrature at the 27 element nodes the stored element matrix is
//   K_e = sum_q w_q detJ_q B_q^T C B_q        (src/preprocess.f90:74-148),
// so K_e p can be formed without K_e: at every GLL point q take the gradient
// of p (each reference derivative is a 3-term sum along one lattice line,
// with the 1D GLL derivative matrix D), map it with J^-1, form the stress
// sigma = C eps with the engineering shears of compute_bmat
// (src/preprocess.f90:12-68) and the isotropic C of compute_cmat
// (src/elastic.f90:13-42), and return it through B_q^T (again 3-term line
// sums).  Per element this reads a 48-byte record per GLL point (J^-1 and the
// three C constants scaled by w_q detJ_q, 1.3 KB per element) instead of the
// 9.7 KB of stored FP32 entries, and costs about 3,600 FMAs per right-hand
// side against 4,617.
//
// Thread (element, node a, trial j): gathers p at node a (combined with z on
// the fly), forms the stress fluxes at GLL point a, then the result rows of
// node a; the element's p and fluxes live in shared memory between the two
// phases.  The FP64 residual of the mixed solve keeps the stored FP64
// matrices, so this operator only steers the FP32 inner iterations.
#include <cstdint>
#include <cstdlib>

#include "sg_kernels.cuh"

namespace sg {

namespace mf {

constexpr int REC = MF_REC;  // floats per GLL point: J^-1 row-major, w detJ c11, w detJ c12, w detJ c44

// D[i][t] = derivative of the 1D Lagrange basis t at GLL point i (nodes -1, 0, 1)
__device__ __forceinline__ constexpr float Dm(int i, int t) {
  return i == 0 ? (t == 0 ? -1.5f : t == 1 ? 2.0f : -0.5f)
                : i == 1 ? (t == 0 ? -0.5f : t == 1 ? 0.0f : 0.5f) : (t == 0 ? 0.5f : t == 1 ? -2.0f : 1.5f);
}

template <int KR>
struct Shape {
  static constexpr int TPE = NGLL * KR;                       // threads per element
  static constexpr int EPC = TPE >= 216 ? 1 : 216 / TPE;      // elements per CTA
  static constexpr int NT = ((EPC * TPE + 31) / 32) * 32;     // CTA threads
  static constexpr int UF = NEDOF * KR;                       // p values per element
  static constexpr int SF = NGLL * 9 * KR;                    // flux values per element
};

// Gradient of the three components along the lattice lines through point a:
// g[c][r] = sum_t D[i_r][t] u_c(node with index t in direction r).
template <int KR>
__device__ __forceinline__ void ref_grad(const float* __restrict__ U, int a, int j, float g[3][3]) {
  const int ic[3] = {a % 3, (a / 3) % 3, a / 9};
  const int st[3] = {1, 3, 9};
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int base = a - ic[r] * st[r];
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      const float d = Dm(ic[r], t);
      const float* u = U + (size_t)(3 * (base + t * st[r])) * KR + j;
      s0 = fmaf(d, u[0], s0);
      s1 = fmaf(d, u[KR], s1);
      s2 = fmaf(d, u[2 * KR], s2);
    }
    g[0][r] = s0;
    g[1][r] = s1;
    g[2][r] = s2;
  }
}

template <int KR>
__global__ void __launch_bounds__(Shape<KR>::NT) k_apply_mf(
    const float* __restrict__ rec, const int* __restrict__ ge, int nelmt, const float* __restrict__ pold,
    const float* __restrict__ z, int combine, float* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ pos) {
  using S = Shape<KR>;
  if (G && G->all_done) return;
  __shared__ __align__(16) float sU[S::EPC][S::UF];
  __shared__ __align__(16) float sS[S::EPC][S::SF];
  const int t = threadIdx.x;
  const int el = t / S::TPE, rem = t - el * S::TPE;
  const int a = rem / KR, j = rem - a * KR;
  const bool act = el < S::EPC;
  const float beta = (act && combine) ? (float)cs[j].beta : 0.f;
  float* U = sU[act ? el : 0];
  float* F = sS[act ? el : 0];
  const int estride = gridDim.x * S::EPC;
  // software pipeline: the next element's dof numbers arrive during this
  // element's first phase and its p and z values during the second, so the
  // global-memory latency overlaps the shared-memory arithmetic
  auto load_dofs = [&](int e, int (&gd)[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) gd[c] = (act && e < nelmt) ? __ldg(ge + (size_t)e * NEDOF + 3 * a + c) : 0;
  };
  auto load_p = [&](const int (&gd)[3], float (&pv)[3], float (&zv)[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pv[c] = pold[(size_t)gd[c] * KR + j];
      zv[c] = combine ? z[(size_t)gd[c] * KR + j] : 0.f;
    }
  };
  int e = blockIdx.x * S::EPC + el;
  int gd[3];
  float pv[3], zv[3];
  load_dofs(e, gd);
  load_p(gd, pv, zv);
  for (int e0 = blockIdx.x * S::EPC; e0 < nelmt; e0 += estride, e += estride) {
    const bool valid = act && e < nelmt;
    if (act) {
#pragma unroll
      for (int c = 0; c < 3; ++c) U[(3 * a + c) * KR + j] = valid ? (combine ? fmaf(beta, pv[c], zv[c]) : pv[c]) : 0.f;
    }
    int gdn[3];
    load_dofs(e + estride, gdn);
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
    int q = -1;
    if (valid) {
      const float4* R = reinterpret_cast<const float4*>(rec + ((size_t)e * NGLL + a) * REC);
      r0 = __ldg(R);
      r1 = __ldg(R + 1);
      r2 = __ldg(R + 2);
      q = __ldg(pos + (size_t)e * NGLL + a);
    }
    __syncthreads();
    if (valid) {
      float gr[3][3];
      ref_grad<KR>(U, a, j, gr);
      const float Ji[9] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x};
      const float c11 = r2.y, c12 = r2.z, c44 = r2.w;
      // physical gradient gp[c][d] = du_c/dx_d = sum_r Ji[3d+r] gr[c][r]
      float gp[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          gp[c][d] = fmaf(Ji[3 * d], gr[c][0], fmaf(Ji[3 * d + 1], gr[c][1], Ji[3 * d + 2] * gr[c][2]));
      // stress (already weighted by w detJ): normal from c11, c12; shears c44 x engineering strain
      const float exx = gp[0][0], eyy = gp[1][1], ezz = gp[2][2];
      float T[3][3];
      T[0][0] = fmaf(c11, exx, c12 * (eyy + ezz));
      T[1][1] = fmaf(c11, eyy, c12 * (exx + ezz));
      T[2][2] = fmaf(c11, ezz, c12 * (exx + eyy));
      T[0][1] = T[1][0] = c44 * (gp[0][1] + gp[1][0]);
      T[1][2] = T[2][1] = c44 * (gp[1][2] + gp[2][1]);
      T[0][2] = T[2][0] = c44 * (gp[0][2] + gp[2][0]);
      // fluxes F[c][r] = sum_d Ji[3d+r] T[c][d]
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          F[((3 * a + c) * 3 + r) * KR + j] =
              fmaf(Ji[r], T[c][0], fmaf(Ji[3 + r], T[c][1], Ji[6 + r] * T[c][2]));
    }
    load_p(gdn, pv, zv);
    __syncthreads();
    if (valid) {
      // rows of node a: y_c(a) = sum_r sum_t D[t][i_r(a)] F_(point t on line r)[c][r]
      const int ic[3] = {a % 3, (a / 3) % 3, a / 9};
      const int st[3] = {1, 3, 9};
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const int base = a - ic[r] * st[r];
#pragma unroll
        for (int tt = 0; tt < 3; ++tt) {
          const float d = Dm(tt, ic[r]);
          const float* f = F + (size_t)((3 * (base + tt * st[r])) * 3 + r) * KR + j;
          y0 = fmaf(d, f[0], y0);
          y1 = fmaf(d, f[3 * KR], y1);
          y2 = fmaf(d, f[6 * KR], y2);
        }
      }
      if (q >= 0) {
        float* dst = Y + (size_t)q * 3 * KR + j;
        dst[0] = y0;
        dst[KR] = y1;
        dst[2 * KR] = y2;
      }
    }
    __syncthreads();
  }
}

// Stress fluxes at one GLL point from the reference gradient gr[c][r] and the
// point record (J^-1, w detJ C): F[c][r] = sum_d Ji[3d+r] T[c][d].
__device__ __forceinline__ void point_flux(const float4 r0, const float4 r1, const float4 r2, const float (&gr)[3][3],
                                           float (&F)[3][3]) {
  const float Ji[9] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x};
  const float c11 = r2.y, c12 = r2.z, c44 = r2.w;
  float gp[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      gp[c][d] = fmaf(Ji[3 * d], gr[c][0], fmaf(Ji[3 * d + 1], gr[c][1], Ji[3 * d + 2] * gr[c][2]));
  const float exx = gp[0][0], eyy = gp[1][1], ezz = gp[2][2];
  float T[3][3];
  T[0][0] = fmaf(c11, exx, c12 * (eyy + ezz));
  T[1][1] = fmaf(c11, eyy, c12 * (exx + ezz));
  T[2][2] = fmaf(c11, ezz, c12 * (exx + eyy));
  T[0][1] = T[1][0] = c44 * (gp[0][1] + gp[1][0]);
  T[1][2] = T[2][1] = c44 * (gp[1][2] + gp[2][1]);
  T[0][2] = T[2][0] = c44 * (gp[0][2] + gp[2][0]);
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) F[c][r] = fmaf(Ji[r], T[c][0], fmaf(Ji[3 + r], T[c][1], Ji[6 + r] * T[c][2]));
}

// Line form of the same operator: thread (element, xi-line (iy, iz), trial j)
// owns the line's three nodes and GLL points.  The xi derivatives and the xi
// fluxes stay in registers; only the eta and zeta terms go through shared
// memory (2/3 of the shared traffic of the point form).  The arithmetic and
// its order are those of k_apply_mf, so the results are bitwise equal.
template <int KR>
struct LShape {
  static constexpr int TPE = 9 * KR;                          // threads per element
  static constexpr int EPC = TPE >= 224 ? 1 : 224 / TPE;      // elements per CTA
  static constexpr int NT = ((EPC * TPE + 31) / 32) * 32;
  static constexpr int UF = NEDOF * KR;                       // p per element [node][c][j]
  static constexpr int SF = NGLL * 6 * KR;                    // eta, zeta fluxes [point][c][2][j]
};

template <int KR>
__global__ void __launch_bounds__(LShape<KR>::NT, 2) k_apply_mf_lines(
    const float* __restrict__ rec, const int* __restrict__ ge, int nelmt, const float* __restrict__ pold,
    const float* __restrict__ z, int combine, float* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ pos) {
  using S = LShape<KR>;
  if (G && G->all_done) return;
  __shared__ __align__(16) float sU[S::EPC][S::UF];
  __shared__ __align__(16) float sS[S::EPC][S::SF];
  const int t = threadIdx.x;
  const int el = t / S::TPE, rem = t - el * S::TPE;
  const int line = rem / KR, j = rem - line * KR;
  const int iy = line % 3, iz = line / 3;
  const int nbase = 3 * iy + 9 * iz;  // node ix = 0 of the line
  const bool act = el < S::EPC;
  const float beta = (act && combine) ? (float)cs[j].beta : 0.f;
  float* U = sU[act ? el : 0];
  float* Fs = sS[act ? el : 0];
  const int estride = gridDim.x * S::EPC;
  int e = blockIdx.x * S::EPC + el;
  // software pipeline as in k_apply_mf: next element's dof numbers during the
  // first phase, its p and z rows during the second
  int gd[9];
  float pv[9], zv[9];
  auto load_dofs = [&](int ee, int (&g)[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k)
      g[k] = (act && ee < nelmt) ? __ldg(ge + (size_t)ee * NEDOF + 3 * nbase + k) : 0;
  };
  auto load_p = [&](const int (&g)[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      pv[k] = pold[(size_t)g[k] * KR + j];
      zv[k] = combine ? z[(size_t)g[k] * KR + j] : 0.f;
    }
  };
  load_dofs(e, gd);
  load_p(gd);
  for (int e0 = blockIdx.x * S::EPC; e0 < nelmt; e0 += estride, e += estride) {
    const bool valid = act && e < nelmt;
    float uR[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float u = valid ? (combine ? fmaf(beta, pv[3 * i + c], zv[3 * i + c]) : pv[3 * i + c]) : 0.f;
        uR[i][c] = u;
        if (act) U[(3 * (nbase + i) + c) * KR + j] = u;
      }
    int gdn[9];
    load_dofs(e + estride, gdn);
    __syncthreads();
    float Fx[3][3];  // xi fluxes of the line's points [i][c]
    if (valid) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int q = nbase + i;
        const float4* R = reinterpret_cast<const float4*>(rec + ((size_t)e * NGLL + q) * REC);
        const float4 r0 = __ldg(R), r1 = __ldg(R + 1), r2 = __ldg(R + 2);
        float gr[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
          for (int tt = 0; tt < 3; ++tt) {
            sx = fmaf(Dm(i, tt), uR[tt][c], sx);
            sy = fmaf(Dm(iy, tt), U[(3 * (i + 3 * tt + 9 * iz) + c) * KR + j], sy);
            sz = fmaf(Dm(iz, tt), U[(3 * (i + 3 * iy + 9 * tt) + c) * KR + j], sz);
          }
          gr[c][0] = sx;
          gr[c][1] = sy;
          gr[c][2] = sz;
        }
        float F[3][3];
        point_flux(r0, r1, r2, gr, F);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          Fx[i][c] = F[c][0];
          Fs[((3 * q + c) * 2 + 0) * KR + j] = F[c][1];
          Fs[((3 * q + c) * 2 + 1) * KR + j] = F[c][2];
        }
      }
    }
    load_p(gdn);
    __syncthreads();
    if (valid) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int n = nbase + i;
        float y[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float acc = 0.f;
#pragma unroll
          for (int tt = 0; tt < 3; ++tt) acc = fmaf(Dm(tt, i), Fx[tt][c], acc);
#pragma unroll
          for (int tt = 0; tt < 3; ++tt) acc = fmaf(Dm(tt, iy), Fs[((3 * (i + 3 * tt + 9 * iz) + c) * 2 + 0) * KR + j], acc);
#pragma unroll
          for (int tt = 0; tt < 3; ++tt) acc = fmaf(Dm(tt, iz), Fs[((3 * (i + 3 * iy + 9 * tt) + c) * 2 + 1) * KR + j], acc);
          y[c] = acc;
        }
        const int q = __ldg(pos + (size_t)e * NGLL + n);
        if (q >= 0) {
          float* dst = Y + (size_t)q * 3 * KR + j;
          dst[0] = y[0];
          dst[KR] = y[1];
          dst[2 * KR] = y[2];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) gd[k] = gdn[k];
    __syncthreads();
  }
}

// Record of GLL point q of operator element le (element elist[le]):
// J^-1 (row-major, as cached by the geometry kernel) and the compute_cmat
// constants times w_q detJ_q, rounded to FP32.
__global__ void k_mf_record(const double* __restrict__ geo, const int* __restrict__ mat_id,
                            const int* __restrict__ elist, int nel, const double* __restrict__ ym,
                            const double* __restrict__ nu, float* __restrict__ rec) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nel * NGLL) return;
  const int le = tid / NGLL, q = tid - le * NGLL;
  const int e = elist ? elist[le] : le;
  const int im = mat_id[e] - 1;
  const double E = ym[im], v = nu[im];
  const double onepv = 1.0 + v, onemv = 1.0 - v, onem2v = 1.0 - 2.0 * v;
  const double Ef = E / (onepv * onem2v);
  const double w1[3] = {1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0};
  const double* g = geo + ((size_t)e * NGLL + q) * GEO_STRIDE;
  const double wd = w1[q % 3] * w1[(q / 3) % 3] * w1[q / 9] * g[9];
  float* r = rec + ((size_t)le * NGLL + q) * REC;
#pragma unroll
  for (int i = 0; i < 9; ++i) r[i] = (float)g[i];
  r[9] = (float)(wd * onemv * Ef);
  r[10] = (float)(wd * v * Ef);
  r[11] = (float)(wd * 0.5 * onem2v * Ef);
}

}  // namespace mf

template <int KR>
void launch_apply_mf(const float* rec, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                     float* Y, const ColState* cs, const PcgGlobal* G, const int* pos, cudaStream_t s) {
  static const bool lines = !getenv("SG_MF_POINTS");
  if (lines) {
    using S = mf::LShape<KR>;
    const int nb = (nelmt + S::EPC - 1) / S::EPC;
    const int grid = nb < 152 * 8 ? nb : 152 * 8;
    if (grid < 1) return;
    mf::k_apply_mf_lines<KR><<<grid, S::NT, 0, s>>>(rec, ge, nelmt, pold, z, combine, Y, cs, G, pos);
    return;
  }
  using S = mf::Shape<KR>;
  const int nb = (nelmt + S::EPC - 1) / S::EPC;
  const int grid = nb < 152 * 8 ? nb : 152 * 8;
  if (grid < 1) return;
  mf::k_apply_mf<KR><<<grid, S::NT, 0, s>>>(rec, ge, nelmt, pold, z, combine, Y, cs, G, pos);
}

void launch_mf_record(const double* geo, const int* mat_id, const int* elist, int nel, const double* ym,
                      const double* nu, float* rec, cudaStream_t s) {
  if (nel <= 0 || !rec) return;
  const int n = nel * NGLL;
  mf::k_mf_record<<<(n + 255) / 256, 256, 0, s>>>(geo, mat_id, elist, nel, ym, nu, rec);
}

template void launch_apply_mf<1>(const float*, const int*, int, const float*, const float*, int, float*,
                                 const ColState*, const PcgGlobal*, const int*, cudaStream_t);
template void launch_apply_mf<2>(const float*, const int*, int, const float*, const float*, int, float*,
                                 const ColState*, const PcgGlobal*, const int*, cudaStream_t);
template void launch_apply_mf<4>(const float*, const int*, int, const float*, const float*, int, float*,
                                 const ColState*, const PcgGlobal*, const int*, cudaStream_t);
template void launch_apply_mf<8>(const float*, const int*, int, const float*, const float*, int, float*,
                                 const ColState*, const PcgGlobal*, const int*, cudaStream_t);
template void launch_apply_mf<16>(const float*, const int*, int, const float*, const float*, int, float*,
                                  const ColState*, const PcgGlobal*, const int*, cudaStream_t);

}  // namespace sg
