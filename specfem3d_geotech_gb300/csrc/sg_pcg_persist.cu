// sg_pcg_persist.cu -- the FP32 PCG iterations of small meshes as one
// persistent cooperative kernel.
//
// On a few thousand elements a PCG iteration (element apply, gather, vector
// update) does about a microsecond of work but costs three dependent kernels,
// each a chain of global-memory round trips plus a last-block reduction.
// Here a chunk of iterations runs inside one cooperative launch: the three
// phases of an iteration are separated by a grid barrier, and instead of a
// last block every block recomputes alpha (after the gather) and the stop
// test and beta (after the update) from the block partials, in the same fixed
// order, so all blocks agree without another barrier and the results are
// deterministic.  Data written by another block in the same launch is read
// through L2 (ld.global.cg).
//
// The phases do the arithmetic of the separate kernels: the matrix-free
// element apply with p = z + beta p_old formed on the fly (sg_apply_mf.cu),
// the gather of element products in element order fused with p = z + beta p
// and the compensated p.kp partials, and u += alpha p, r -= alpha kp,
// z = D r with the max-norms and compensated r.z, r.r partials; the
// per-column stop tests are those of the update kernel (reference step test
// of src/solver.f90:61-73 or the residual-reduction test).
//
// The barrier is bounded: a block that waits too long sets the error word of
// the solve's control word and leaves; every other block's wait then runs out
// as well, the launch ends and the solve reports SG_ERR_TIMEOUT without
// launching another chunk.  The barrier's arrival count and generation live in
// the solve's own control word (the count is zeroed before every launch), so
// concurrent solves on other streams do not share them.
#include <cstdint>
#include <cstdlib>

#include "sg_kernels.cuh"

namespace sg {

namespace pp {

constexpr int NT = 256;               // threads per block
constexpr int BAR_TRIES = 1 << 20;    // bounded barrier wait (x ~64 ns)

// compensated FP32 dot accumulator (exact products, two-float sum)
struct CompSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b, e = fmaf(a, b, -p);
    const float t = hi + p, bp = t - hi;
    const float err = (hi - (t - bp)) + (p - bp);
    hi = t;
    lo += err + e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ float ldf(const float* p) { return __ldcg(p); }

// Grid barrier on (count = G->cntB, generation = G->pad).  Returns false (for
// every thread of the block) when the wait ran out.
__device__ __forceinline__ bool grid_barrier(PcgGlobal* G) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &G->pad;
    const unsigned g0 = *gen;
    __threadfence();
    if (atomicAdd(&G->cntB, 1u) == gridDim.x - 1) {
      atomicExch(&G->cntB, 0u);
      __threadfence();
      atomicAdd(&G->pad, 1u);
    } else {
      int tries = 0;
      while (*gen == g0) {
        if (++tries > BAR_TRIES) {
          ok = 0;
          atomicExch(&G->err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  return __syncthreads_and(threadIdx.x != 0 || ok) != 0;
}

__device__ __forceinline__ constexpr float Dm(int i, int t) {
  return i == 0 ? (t == 0 ? -1.5f : t == 1 ? 2.0f : -0.5f)
                : i == 1 ? (t == 0 ? -0.5f : t == 1 ? 0.0f : 0.5f) : (t == 0 ? 0.5f : t == 1 ? -2.0f : 1.5f);
}

struct Args {
  const float* rec;   // matrix-free point records (MF_REC floats per GLL point)
  const int* ge;      // dof map of the operator elements
  int nelmt;
  const int* pos;     // gather position of each element slot
  const int* gptr;    // gather groups: slot range and dof numbers
  const int* gdof;
  int ngroups;
  int n1;
  float *u, *r, *z, *p, *kp, *Y;
  const float* dp;    // inverted diagonal
  ColState* cs;
  PcgGlobal* G;
  double* part;       // gather partials [grid][KR], update partials [grid][KR][4]
  int chunk;          // iterations to run
};

template <int KR>
struct Shape {
  static constexpr int TPE = NGLL * KR;
  static constexpr int EPC = NT / TPE;         // elements per block pass of the apply
  static constexpr int UF = NEDOF * KR;
  static constexpr int SF = NGLL * 9 * KR;
};

template <int KR>
__global__ void __launch_bounds__(NT, 4) k_pcg_persistent(Args A) {
  using S = Shape<KR>;
  static_assert(S::EPC >= 1, "KR up to 8");
  __shared__ __align__(16) float sU[S::EPC][S::UF];
  __shared__ __align__(16) float sF[S::EPC][S::SF];
  __shared__ double sred[NT / 32][KR][4];
  __shared__ double sfin[NT];
  // block-local copy of the column state (identical in every block)
  __shared__ double c_rz[KR], c_alpha[KR], c_beta[KR], c_tol[KR], c_rr0[KR], c_maxp[KR], c_maxu[KR], c_rr[KR];
  __shared__ int c_active[KR], c_done[KR], c_iters[KR], c_failed[KR];
  __shared__ int s_it, s_alldone;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  PcgGlobal* G = A.G;
  if (G->all_done) return;
  if (t < KR) {
    const ColState c = A.cs[t];
    c_rz[t] = c.rz; c_alpha[t] = c.alpha; c_beta[t] = c.beta; c_tol[t] = c.tol; c_rr0[t] = c.rr0;
    c_maxp[t] = c.maxp; c_maxu[t] = c.maxu; c_rr[t] = c.rr;
    c_active[t] = c.active; c_done[t] = c.done; c_iters[t] = c.iters; c_failed[t] = c.failed;
  }
  if (t == 0) { s_it = G->it; s_alldone = 0; }
  const int maxiter = G->maxiter, mode = G->mode, kcols = G->kcols;
  __syncthreads();
  const int grid = gridDim.x;
  double* partg = A.part;                          // [grid][KR]
  double* partu = A.part + (size_t)grid * KR;      // [grid][KR][4]
  // apply-phase thread mapping: element slot el, node a, column j
  const int el = t / S::TPE, rem = t - el * S::TPE;
  const int a = rem / KR, ja = rem - a * KR;
  const bool act = el < S::EPC;
  float* U = sU[act ? el : 0];
  float* F = sF[act ? el : 0];
  // gather / update mapping: the column of a thread is fixed (NT % KR == 0)
  const int jt = t % KR;

  for (int k = 0; k < A.chunk; ++k) {
    // ---- phase A: element products of p = z + beta p_old (matrix-free) ----
    {
      const float beta = act ? (float)c_beta[ja] : 0.f;
      const int estride = grid * S::EPC;
      // software pipeline: the next element's p and z values load while this
      // element computes (its dof numbers one element further ahead)
      int e = blockIdx.x * S::EPC + el;
      int gd[3], gdn[3];
      float pv[3], zv[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) gd[c] = (act && e < A.nelmt) ? __ldg(A.ge + (size_t)e * NEDOF + 3 * a + c) : 0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pv[c] = ldf(A.p + (size_t)gd[c] * KR + ja);
        zv[c] = ldf(A.z + (size_t)gd[c] * KR + ja);
      }
      for (int e0 = blockIdx.x * S::EPC; e0 < A.nelmt; e0 += estride, e += estride) {
        const bool valid = act && e < A.nelmt;
        if (act) {
#pragma unroll
          for (int c = 0; c < 3; ++c) U[(3 * a + c) * KR + ja] = valid ? fmaf(beta, pv[c], zv[c]) : 0.f;
        }
        const int en = e + estride;
#pragma unroll
        for (int c = 0; c < 3; ++c) gdn[c] = (act && en < A.nelmt) ? __ldg(A.ge + (size_t)en * NEDOF + 3 * a + c) : 0;
        __syncthreads();
        if (valid) {
          const int ic[3] = {a % 3, (a / 3) % 3, a / 9};
          const int st[3] = {1, 3, 9};
          float gr[3][3];
#pragma unroll
          for (int rr = 0; rr < 3; ++rr) {
            const int base = a - ic[rr] * st[rr];
            float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int tt = 0; tt < 3; ++tt) {
              const float d = Dm(ic[rr], tt);
              const float* uu = U + (size_t)(3 * (base + tt * st[rr])) * KR + ja;
              s0 = fmaf(d, uu[0], s0);
              s1 = fmaf(d, uu[KR], s1);
              s2 = fmaf(d, uu[2 * KR], s2);
            }
            gr[0][rr] = s0; gr[1][rr] = s1; gr[2][rr] = s2;
          }
          const float4* R = reinterpret_cast<const float4*>(A.rec + ((size_t)e * NGLL + a) * MF_REC);
          const float4 r0 = __ldg(R), r1 = __ldg(R + 1), r2 = __ldg(R + 2);
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
            for (int rr = 0; rr < 3; ++rr)
              F[((3 * a + c) * 3 + rr) * KR + ja] =
                  fmaf(Ji[rr], T[c][0], fmaf(Ji[3 + rr], T[c][1], Ji[6 + rr] * T[c][2]));
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          pv[c] = ldf(A.p + (size_t)gdn[c] * KR + ja);
          zv[c] = ldf(A.z + (size_t)gdn[c] * KR + ja);
        }
        __syncthreads();
        if (valid) {
          const int ic[3] = {a % 3, (a / 3) % 3, a / 9};
          const int st[3] = {1, 3, 9};
          float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
          for (int rr = 0; rr < 3; ++rr) {
            const int base = a - ic[rr] * st[rr];
#pragma unroll
            for (int tt = 0; tt < 3; ++tt) {
              const float d = Dm(tt, ic[rr]);
              const float* f = F + (size_t)((3 * (base + tt * st[rr])) * 3 + rr) * KR + ja;
              y0 = fmaf(d, f[0], y0);
              y1 = fmaf(d, f[3 * KR], y1);
              y2 = fmaf(d, f[6 * KR], y2);
            }
          }
          const int q = __ldg(A.pos + (size_t)e * NGLL + a);
          if (q >= 0) {
            float* dst = A.Y + (size_t)q * 3 * KR + ja;
            dst[0] = y0;
            dst[KR] = y1;
            dst[2 * KR] = y2;
          }
        }
        __syncthreads();
      }
    }
    if (!grid_barrier(G)) return;

    // ---- phase B: kp = sum of the element products in element order; p = z + beta p ----
    {
      const bool live = c_active[jt] && !c_done[jt];
      const float beta = (float)c_beta[jt];
      CompSum dot;
      const size_t items = (size_t)A.ngroups * 3 * KR;
      for (size_t it = (size_t)blockIdx.x * NT + t; it < items; it += (size_t)grid * NT) {
        const int g = (int)(it / (3 * KR)), c = (int)(it - (size_t)g * 3 * KR), d = c / KR;
        const int s0 = __ldg(A.gptr + g), s1 = __ldg(A.gptr + g + 1);
        float acc = 0.f;
        for (int sl = s0; sl < s1; ++sl) acc = acc + ldf(A.Y + (size_t)sl * 3 * KR + c);
        const int gd = __ldg(A.gdof + 3 * g + d);
        if (!gd) continue;
        float* pp = A.p + (size_t)gd * KR + jt;
        if (live) {
          const float pv = fmaf(beta, ldf(pp), ldf(A.z + (size_t)gd * KR + jt));
          dot.add(pv, acc);
          *pp = pv;
        }
        A.kp[(size_t)gd * KR + jt] = acc;
      }
      double v = dot.value();
#pragma unroll
      for (int o = 16; o >= KR; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane < KR) sred[warp][lane][0] = v;
      __syncthreads();
      if (t < KR) {
        double s = 0.0;
        for (int w = 0; w < NT / 32; ++w) s += sred[w][t][0];
        partg[(size_t)blockIdx.x * KR + t] = s;
      }
    }
    if (!grid_barrier(G)) return;
    // alpha = r.z / p.kp, the block partials summed in a fixed order
    {
      double v = 0.0;
      for (int b = t / KR; b < grid; b += NT / KR) v += __ldcg(partg + (size_t)b * KR + jt);
      sfin[t] = v;
      __syncthreads();
      if (t < KR) {
        double s = 0.0;
        for (int u = t; u < NT; u += KR) s += sfin[u];
        if (c_active[t] && !c_done[t]) c_alpha[t] = c_rz[t] / s;
      }
      __syncthreads();
    }

    // ---- phase C: u += alpha p, r -= alpha kp, z = D r, norms and dots ----
    {
      const bool live = c_active[jt] && !c_done[jt];
      const float alpha = (float)c_alpha[jt];
      float mp = 0.f, mu = 0.f;
      CompSum rz, rr;
      if (live) {
        const size_t items = (size_t)A.n1 * KR;
        for (size_t i = (size_t)blockIdx.x * NT + t; i < items; i += (size_t)grid * NT) {
          const float pv = ldf(A.p + i), uv = ldf(A.u + i), rv = ldf(A.r + i), kv = ldf(A.kp + i);
          const float un = fmaf(alpha, pv, uv);
          const float rn = fmaf(-alpha, kv, rv);
          const float zn = __ldg(A.dp + i / KR) * rn;
          A.u[i] = un;
          A.r[i] = rn;
          A.z[i] = zn;
          mp = fmaxf(mp, fabsf(pv));
          mu = fmaxf(mu, fabsf(un));
          rz.add(rn, zn);
          rr.add(rn, rn);
        }
      }
      double q4[4] = {(double)mp, (double)mu, live ? rz.value() : 0.0, live ? rr.value() : 0.0};
#pragma unroll
      for (int o = 16; o >= KR; o >>= 1) {
        q4[0] = fmax(q4[0], __shfl_xor_sync(0xffffffffu, q4[0], o));
        q4[1] = fmax(q4[1], __shfl_xor_sync(0xffffffffu, q4[1], o));
        q4[2] += __shfl_xor_sync(0xffffffffu, q4[2], o);
        q4[3] += __shfl_xor_sync(0xffffffffu, q4[3], o);
      }
      if (lane < KR)
#pragma unroll
        for (int q = 0; q < 4; ++q) sred[warp][lane][q] = q4[q];
      __syncthreads();
      if (t < 4 * KR) {
        const int j = t / 4, q = t % 4;
        double s = 0.0;
        for (int w = 0; w < NT / 32; ++w) s = (q < 2) ? fmax(s, sred[w][j][q]) : s + sred[w][j][q];
        partu[((size_t)blockIdx.x * KR + j) * 4 + q] = s;
      }
    }
    if (!grid_barrier(G)) return;
    // stop tests and beta, identical in every block
    {
      constexpr int NQ = 4 * KR;
      const int q = t % 4;
      double v = 0.0;
      for (int idx = t; idx < grid * NQ; idx += NT) {
        const double x = __ldcg(partu + idx);
        v = (q < 2) ? fmax(v, x) : v + x;
      }
      sfin[t] = v;
      __syncthreads();
      const int itn = s_it + 1;
      if (t == 0) s_alldone = 1;
      __syncthreads();
      if (t < KR) {
        double amax = 0.0, bmax = 0.0, s = 0.0, qq = 0.0;
        for (int u = t * 4; u < NT; u += NQ) {
          amax = fmax(amax, sfin[u]); bmax = fmax(bmax, sfin[u + 1]); s += sfin[u + 2]; qq += sfin[u + 3];
        }
        if (c_active[t] && !c_done[t]) {
          c_maxp[t] = amax; c_maxu[t] = bmax; c_rr[t] = qq;
          const bool stop = ((mode & 1) == 0) ? (fabs(c_alpha[t]) * amax / bmax <= c_tol[t])
                                              : (qq <= c_tol[t] * c_tol[t] * c_rr0[t]);
          if (stop) {
            c_done[t] = 1; c_iters[t] = itn;
          } else if (itn >= maxiter) {
            c_done[t] = 1; c_failed[t] = 1; c_iters[t] = maxiter + 1;
          } else {
            c_beta[t] = s / c_rz[t];
            c_rz[t] = s;
          }
        }
        if (t < kcols && c_active[t] && !c_done[t]) atomicAnd(&s_alldone, 0);
      }
      __syncthreads();
      if (t == 0) s_it = itn;
      __syncthreads();
      if (s_alldone) break;
    }
  }
  // the column state leaves with block 0
  if (blockIdx.x == 0) {
    if (t < KR) {
      ColState& c = A.cs[t];
      c.rz = c_rz[t]; c.alpha = c_alpha[t]; c.beta = c_beta[t]; c.maxp = c_maxp[t]; c.maxu = c_maxu[t];
      c.rr = c_rr[t]; c.done = c_done[t]; c.iters = c_iters[t]; c.failed = c_failed[t];
    }
    if (t == 0) {
      G->it = s_it;
      G->all_done = s_alldone;
    }
  }
}

template <int KR>
int max_blocks() {
  static int per_sm = -1;
  if (per_sm < 0) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pcg_persistent<KR>, NT, 0) != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    per_sm = n;
  }
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return per_sm * nsm;
}

}  // namespace pp

// Per PCG iteration with 8 trials, persistent against separate kernels:
// 22.7 against 34.2 us at 270 elements, 33.5 against 39.9 at 1,125; at 3,000
// and above the separate kernels are as fast or faster.
int persist_max_elements() { return 1500; }

bool persist_enabled() {
  static const bool on = !(getenv("SG_PERSIST") && atoi(getenv("SG_PERSIST")) == 0);
  return on;
}

// Runs `chunk` PCG iterations of the FP32 solve as one cooperative launch.
// Returns false when the launch is not possible (the caller then runs the
// separate kernels).
template <int KR>
bool launch_pcg_persistent(const float* rec, const int* ge, int nelmt, const int* pos, const GatherTopo& T, int n1,
                           float* u, float* r, float* z, float* p, float* kp, float* Y, const float* dp,
                           ColState* cs, PcgGlobal* G, double* part, int chunk, cudaStream_t s) {
  if constexpr (KR > 8) {
    return false;
  } else {
    using S = pp::Shape<KR>;
    int cap = pp::max_blocks<KR>();
    // the barrier's cost grows with the number of blocks: at most one block
    // per SM (33.5 against 36.2 us per iteration with two at 1,125 elements),
    // about four element passes of the apply per block
    if (cap > 152) cap = 152;
    int grid = (nelmt + 4 * S::EPC - 1) / (4 * S::EPC);
    if (grid > cap) grid = cap;
    if (grid < 1) return false;
    // the partial buffer holds NPART * 16 * 4 doubles
    if ((size_t)grid * KR * 5 > (size_t)NPART * 16 * 4) return false;
    // a barrier count left behind by an earlier launch would release the
    // first barrier early: start every launch from zero arrivals
    cudaMemsetAsync(&G->cntB, 0, sizeof(unsigned), s);
    pp::Args A{rec, ge, nelmt, pos, T.d_ptr, T.d_dof, T.ngroups, n1, u, r, z, p, kp, Y, dp, cs, G, part, chunk};
    void* args[] = {&A};
    if (cudaLaunchCooperativeKernel((const void*)pp::k_pcg_persistent<KR>, grid, pp::NT, args, 0, s) !=
        cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    add_launches(1);
    return true;
  }
}

#define SG_PP_INST(KR)                                                                                              \
  template bool launch_pcg_persistent<KR>(const float*, const int*, int, const int*, const GatherTopo&, int, float*, \
                                          float*, float*, float*, float*, float*, const float*, ColState*,          \
                                          PcgGlobal*, double*, int, cudaStream_t);
SG_PP_INST(1)
SG_PP_INST(2)
SG_PP_INST(4)
SG_PP_INST(8)
SG_PP_INST(16)

}  // namespace sg
