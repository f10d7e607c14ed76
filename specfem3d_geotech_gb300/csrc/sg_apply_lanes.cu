// sg_apply_lanes.cu -- batched FP32 element apply, one lane per
// (element, right-hand side).
//
// Y_e[81 x KR] = K_e[81 x 81] P_e[81 x KR] for the KR concurrent SRF trials
// (the element loop of src/solver.f90:53-59, batched over trials).  A warp
// takes EPW = 32/KR consecutive elements; lane (i, j) holds column j of
// element i's P_e and Y_e in registers (81 + 81 floats) and walks the element's
// stored entries in storage order with every index known at compile time:
// a stored off-diagonal node block (n, m) updates both y_n += B p_m and
// y_m += B^T p_n from one read, an own-node block updates y_n only.  All KR
// lanes of an element read the same stored entries, so a 16-byte shared load
// is a broadcast and one wavefront serves the EPW elements of the warp.
//
// The element matrices stream through a per-warp ring of NSTAGE stages; a
// stage holds one 976-byte chunk (61 float4) of each of the warp's elements,
// copied by cp.async.bulk with completion on the stage's mbarrier.  Lane 0
// keeps NSTAGE-1 chunks in flight.  Chunk slots are 976 B apart, so the EPW
// element slots of a stage fall on distinct 16-byte bank groups.  The next
// group's dof numbers and gather positions travel to shared memory by
// cp.async while the current group computes.  Every wait
// is bounded; a timeout sets the caller's error word, the warp drains its own
// copies (bounded) and stops.
//
// Sums per output entry run in storage order, so results are deterministic
// (bitwise equal from run to run) but round differently from the per-node
// order of the node-lane kernels.
#include <cstdint>
#include <utility>

#include "sg_kernels.cuh"

namespace sg {

namespace lanes {

constexpr int NW = 8;          // warps per CTA, one CTA per SM
constexpr int CHF = 244;       // floats per chunk slot (61 float4)
constexpr int NCH = 10;        // chunks per element: 9 x 244 + 236 = KS_STRIDE
constexpr int NSTAGE = 5;      // ring depth; divides NCH so stage and parity are static
constexpr int LAST_F4 = (KS_STRIDE - (NCH - 1) * CHF) / 4;   // 59 float4 in the last chunk
static_assert((NCH - 1) * CHF < KS_STRIDE && NCH * CHF >= KS_STRIDE, "chunking");
static_assert(NCH % NSTAGE == 0, "static stage parity");
static_assert((KS_STRIDE - (NCH - 1) * CHF) % 4 == 0, "16-byte chunk copies");

// Stored node blocks in storage order: for m, for n <= m with (n, m) coupled,
// entries K[3n+c][3m+d] row-major -- the order the stiffness kernel writes.
struct BlockTable {
  unsigned char n[270], m[270];
  int count;
};
constexpr bool coupled(int n, int m) {
  return ((n % 3 != m % 3) + ((n / 3) % 3 != (m / 3) % 3) + (n / 9 != m / 9)) <= 2;
}
constexpr BlockTable make_blocks() {
  BlockTable T{};
  int b = 0;
  for (int m = 0; m < NGLL; ++m)
    for (int n = 0; n <= m; ++n)
      if (coupled(n, m)) {
        T.n[b] = (unsigned char)n;
        T.m[b] = (unsigned char)m;
        ++b;
      }
  T.count = b;
  return T;
}
constexpr BlockTable BT = make_blocks();
static_assert(BT.count * 9 == KS_NNZ, "270 stored node blocks");

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// false if the phase did not complete within the bound
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

// one stored entry T with value v
template <int T>
__device__ __forceinline__ void entry(float v, const float (&p)[NEDOF], float (&y)[NEDOF]) {
  if constexpr (T < KS_NNZ) {
    constexpr int b = T / 9, c = (T % 9) / 3, d = T % 3;
    constexpr int n = BT.n[b], m = BT.m[b];
    y[3 * n + c] = fmaf(v, p[3 * m + d], y[3 * n + c]);
    if constexpr (n != m) y[3 * m + d] = fmaf(v, p[3 * n + c], y[3 * m + d]);
  }
}

template <int C, int... F>
__device__ __forceinline__ void chunk_entries(const float4* __restrict__ src, const float (&p)[NEDOF],
                                              float (&y)[NEDOF], std::integer_sequence<int, F...>) {
  (
      [&] {
        const float4 v = src[F];
        constexpr int T = (C * CHF) + 4 * F;
        entry<T + 0>(v.x, p, y);
        entry<T + 1>(v.y, p, y);
        entry<T + 2>(v.z, p, y);
        entry<T + 3>(v.w, p, y);
      }(),
      ...);
}

template <typename F, int... Cs>
__device__ __forceinline__ void for_chunks(F& f, std::integer_sequence<int, Cs...>) {
  (f(std::integral_constant<int, Cs>{}), ...);
}

constexpr unsigned chunk_bytes(int c) { return (unsigned)(c == NCH - 1 ? LAST_F4 * 16 : CHF * 4); }

constexpr int IDX = NEDOF + NGLL;  // per element: 81 dof numbers + 27 gather positions

template <int KR>
struct Shape {
  static constexpr int EPW = 32 / KR;                       // elements per warp
  static constexpr int STAGE_F = EPW * CHF;                 // floats per stage
  static constexpr int RING_F = NSTAGE * STAGE_F;           // floats per warp ring
  static constexpr int IBUF = 2 * EPW * IDX;                // ints per warp: two groups of indices
  static constexpr int BAR_BYTES = 512;                     // NW * NSTAGE mbarriers, padded
  static constexpr size_t SMEM = BAR_BYTES + (size_t)NW * RING_F * 4 + (size_t)NW * IBUF * 4;
};

__device__ __forceinline__ void cp_async4(int* dst, const int* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// The warp copies group g's dof numbers and gather positions into buf
// (4-byte cp.async, no registers held while they travel).
template <int KR>
__device__ __forceinline__ void prefetch_indices(const int* __restrict__ ge, const int* __restrict__ pos, int nelmt,
                                                 int ngroups, int g, int* buf, int lane) {
  using S = Shape<KR>;
  if (g < ngroups) {
    const int e0 = g * S::EPW;
    const int nv = min(S::EPW, nelmt - e0);
    for (int t = lane; t < nv * IDX; t += 32) {
      const int ii = t / IDX, r = t - ii * IDX;
      const int* src = (r < NEDOF) ? ge + (size_t)(e0 + ii) * NEDOF + r : pos + (size_t)(e0 + ii) * NGLL + (r - NEDOF);
      cp_async4(buf + t, src);
    }
  }
  cp_async_commit();
}

// Lane 0 issues chunk c of group g (all of its valid elements) into stage
// c % NSTAGE; returns false when the group is past the end (nothing issued).
template <int KR>
__device__ __forceinline__ bool issue_chunk(const float* __restrict__ Ks, int nelmt, int ngroups, int g, int c,
                                            float* ring, uint64_t* bar) {
  using S = Shape<KR>;
  if (g >= ngroups) return false;
  const int e0 = g * S::EPW;
  const int nv = min(S::EPW, nelmt - e0);
  const unsigned bytes = chunk_bytes(c);
  float* dst = ring + (c % NSTAGE) * S::STAGE_F;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  expect_tx(bar + (c % NSTAGE), bytes * (unsigned)nv);
  for (int i = 0; i < nv; ++i)
    bulk_copy(dst + i * CHF, Ks + (size_t)(e0 + i) * KS_STRIDE + (size_t)c * CHF, bytes, bar + (c % NSTAGE));
  return true;
}

// The element's direction column (lane j): p_old (MODE 0), beta p_old + z
// (MODE 1), or beta p_old + D (r - alpha kp) with r and kp of the previous
// step (MODE 2, the fused iteration).  Every gather is issued before any is
// combined: the second operand lands in t, the element's accumulators, which
// are free until the products start (and are zeroed here), so all 162 loads
// of a lane are in flight together without registers of their own.
template <int MODE, int KR>
__device__ __forceinline__ void gather_dir(float (&p)[NEDOF], float (&t)[NEDOF], const int* idx, bool valid, int j,
                                           const float* __restrict__ pold, const float* __restrict__ z,
                                           float beta, float alpha, const FusedDir& fz) {
#pragma unroll
  for (int r = 0; r < NEDOF; ++r) {
    const int gd = valid ? idx[r] : 0;
    const size_t o = (size_t)gd * KR + j;
    p[r] = pold[o];
    if constexpr (MODE == 1) t[r] = z[o];
    if constexpr (MODE == 2) t[r] = fz.dinv[gd] * fmaf(-alpha, fz.kp[o], fz.r[o]);
  }
#pragma unroll
  for (int r = 0; r < NEDOF; ++r) {
    float pv = p[r];
    if constexpr (MODE != 0) pv = fmaf(beta, pv, t[r]);
    p[r] = valid ? pv : 0.f;
    t[r] = 0.f;
  }
}

template <int KR, int MODE>
__global__ void __launch_bounds__(NW * 32, 1) k_apply_lanes(
    const float* __restrict__ Ks, const int* __restrict__ ge, int nelmt, const float* __restrict__ pold,
    const float* __restrict__ z, float* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ pos, int* __restrict__ err, FusedDir fz) {
  using S = Shape<KR>;
  if (G && G->all_done) return;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = lane / KR, j = lane % KR;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + warp * NSTAGE;
  float* ring = reinterpret_cast<float*>(smem + S::BAR_BYTES) + (size_t)warp * S::RING_F;
  int* ibuf = reinterpret_cast<int*>(smem + S::BAR_BYTES + (size_t)NW * S::RING_F * 4) + (size_t)warp * S::IBUF;
  const int ngroups = (nelmt + S::EPW - 1) / S::EPW;
  const int gstride = gridDim.x * NW;
  int g = blockIdx.x * NW + warp;
  if (lane == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(bar + s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const float beta = MODE ? (float)cs[j].beta : 0.f;
  const float alpha = MODE == 2 ? (float)cs[j].alpha : 0.f;
  // chunks issued / waited, counted along the warp's chunk sequence
  int issued = 0, waited = 0;
  if (lane == 0)
    for (int c = 0; c < NSTAGE - 1; ++c) issued += issue_chunk<KR>(Ks, nelmt, ngroups, g, c, ring, bar);
  issued = __shfl_sync(0xffffffffu, issued, 0);
  prefetch_indices<KR>(ge, pos, nelmt, ngroups, g, ibuf, lane);
  bool ok = true;
  for (int buf = 0; g < ngroups && ok; g += gstride, buf ^= 1) {
    const int e = g * S::EPW + i;
    const bool valid = e < nelmt;
    // this group's indices have landed; the other buffer (read by the
    // previous group) takes the next group's
    cp_async_wait_all();
    __syncwarp();
    const int* idx = ibuf + buf * (S::EPW * IDX) + i * IDX;
    prefetch_indices<KR>(ge, pos, nelmt, ngroups, g + gstride, ibuf + (buf ^ 1) * (S::EPW * IDX), lane);
    float p[NEDOF], y[NEDOF];
    gather_dir<MODE, KR>(p, y, idx, valid, j, pold, z, beta, alpha, fz);
    const float* mine = ring + i * CHF;
    auto step = [&](auto cc) {
      constexpr int C = decltype(cc)::value;
      if (!ok) return;
      // refill the stage consumed by the previous chunk: chunk C + NSTAGE - 1
      // of this group, or of the warp's next group
      if (lane == 0) {
        constexpr int CN = C + NSTAGE - 1;
        issued += (CN < NCH) ? issue_chunk<KR>(Ks, nelmt, ngroups, g, CN, ring, bar)
                             : issue_chunk<KR>(Ks, nelmt, ngroups, g + gstride, CN - NCH, ring, bar);
      }
      // the verdict is made warp-uniform so that no lane leaves the
      // shared __syncwarp sequence alone
      const bool w = __all_sync(0xffffffffu, mbar_wait(bar + (C % NSTAGE), (unsigned)((C / NSTAGE) & 1)));
      if (!w) {
        if (lane == 0) atomicExch(err, 1);
        ok = false;
        return;
      }
      ++waited;
      const float4* src = reinterpret_cast<const float4*>(mine + (C % NSTAGE) * S::STAGE_F);
      chunk_entries<C>(src, p, y, std::make_integer_sequence<int, (C == NCH - 1) ? LAST_F4 : CHF / 4>{});
      __syncwarp();
    };
    for_chunks(step, std::make_integer_sequence<int, NCH>{});
    if (!ok) break;
    if (valid) {
#pragma unroll
      for (int a = 0; a < NGLL; ++a) {
        const int q = idx[NEDOF + a];
        if (q >= 0) {
          float* dst = Y + (size_t)q * 3 * KR + j;
          dst[0] = y[3 * a];
          dst[KR] = y[3 * a + 1];
          dst[2 * KR] = y[3 * a + 2];
        }
      }
    }
  }
  // drain copies still in flight (after the last group they were never
  // issued; after a timeout this waits, bounded, for the warp's own copies)
  cp_async_wait_all();
  issued = __shfl_sync(0xffffffffu, issued, 0);
  for (int q = waited; q < issued; ++q) mbar_wait(bar + (q % NCH) % NSTAGE, (unsigned)(((q % NCH) / NSTAGE) & 1));
}

}  // namespace lanes

template <int KR>
void launch_apply_lanes(const float* Ks, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                        float* Y, const ColState* cs, const PcgGlobal* G, const int* pos, int* err, cudaStream_t s,
                        FusedDir fz) {
  using S = lanes::Shape<KR>;
  // one kernel per way of forming the direction (separate register budgets)
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(lanes::k_apply_lanes<KR, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    cudaFuncSetAttribute(lanes::k_apply_lanes<KR, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    cudaFuncSetAttribute(lanes::k_apply_lanes<KR, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    attr = true;
  }
  const int ngroups = (nelmt + S::EPW - 1) / S::EPW;
  const int warps = (ngroups + lanes::NW - 1) / lanes::NW;
  int grid = warps < 152 ? warps : 152;
  if (grid < 1) return;
  if (combine == 2)
    lanes::k_apply_lanes<KR, 2><<<grid, lanes::NW * 32, S::SMEM, s>>>(Ks, ge, nelmt, pold, z, Y, cs, G, pos, err, fz);
  else if (combine == 1)
    lanes::k_apply_lanes<KR, 1><<<grid, lanes::NW * 32, S::SMEM, s>>>(Ks, ge, nelmt, pold, z, Y, cs, G, pos, err, fz);
  else
    lanes::k_apply_lanes<KR, 0><<<grid, lanes::NW * 32, S::SMEM, s>>>(Ks, ge, nelmt, pold, z, Y, cs, G, pos, err, fz);
}

size_t apply_lanes_smem(int KR) {
  return KR == 8 ? lanes::Shape<8>::SMEM : KR == 16 ? lanes::Shape<16>::SMEM : lanes::Shape<4>::SMEM;
}

template void launch_apply_lanes<8>(const float*, const int*, int, const float*, const float*, int, float*,
                                    const ColState*, const PcgGlobal*, const int*, int*, cudaStream_t, FusedDir);
template void launch_apply_lanes<16>(const float*, const int*, int, const float*, const float*, int, float*,
                                     const ColState*, const PcgGlobal*, const int*, int*, cudaStream_t, FusedDir);

}  // namespace sg
