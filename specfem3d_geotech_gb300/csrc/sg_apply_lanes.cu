// sg_apply_lanes.cu -- batched FP32 element apply, one lane per
// (element, right-hand side).
//
// Y_e[81 x KR] = K_e[81 x 81] P_e[81 x KR] for the KR concurrent SRF trials
// (the element loop of src/solver.f90:53-59, batched over trials).  A warp
// takes EPW = 32/KR consecutive elements; lane (i, j) holds column j of
// element i's P_e and Y_e in registers and walks the element's stored entries
// with every index known at compile time: a stored off-diagonal node block
// (n, m) updates both y_n += B p_m and y_m += B^T p_n from one read, an
// own-node block updates y_n only.  All KR lanes of an element read the same
// stored entries, so a 16-byte shared load is a broadcast and one wavefront
// serves the EPW elements of the warp.
//
// The walk goes down the columns (m = 26 .. 0, see Traversal): a node's rows
// are complete, and its p values dead, as soon as its column is done, so its
// three rows are stored there and the freed registers take the next group's p
// and z values of that node -- the gather of the next group overlaps this
// group's arithmetic instead of stalling the warp at the group's start.
//
// The element matrices stream through a per-warp ring of NSTAGE stages; a
// stage holds one 976-byte chunk (61 float4) of each of the warp's elements,
// copied by cp.async.bulk with completion on the stage's mbarrier, in walk
// order (last chunk first).  Lane 0 keeps NSTAGE-1 chunks in flight.  Chunk
// slots are 976 B apart, so the EPW element slots of a stage fall on distinct
// 16-byte bank groups.  Dof numbers and gather positions travel to shared
// memory by cp.async two groups ahead.  Every wait is bounded; a timeout sets
// the caller's error word, the warp drains its own copies (bounded) and
// stops.
//
// Sums per output entry run in the walk order, so results are deterministic
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

// Traversal order.  Columns (node m of a stored block (n, m), n <= m) are
// walked from m = 26 down to 0, the stored entries in reverse storage order.
// Block (n, m) adds K p_m to y_n and K^T p_n to y_m; y_m also receives K p_m'
// from the blocks (m, m') of the columns m' > m.  Walking columns downwards,
// y_m is therefore complete, and p_m no longer needed, right after column m:
// its three rows are stored at once and the freed registers receive the next
// group's p and z values of node m.  The loads of the next group thus travel
// during this group's arithmetic, and the register footprint stays level.
struct Traversal {
  int col_first[NGLL];      // first stored entry (storage order) of column m
  short done_col[KS_NNZ];   // m when entry T is column m's first entry, else -1
  bool first_a[KS_NNZ];     // the update of y_n by entry T is the row's first (walking down)
  bool first_b[KS_NNZ];     // the same for the transposed update of y_m
};
constexpr Traversal make_traversal() {
  Traversal R{};
  for (int m = 0; m < NGLL; ++m) R.col_first[m] = -1;
  for (int b = 0; b < BT.count; ++b)
    if (R.col_first[BT.m[b]] < 0) R.col_first[BT.m[b]] = 9 * b;
  for (int T = 0; T < KS_NNZ; ++T) R.done_col[T] = -1;
  for (int m = 0; m < NGLL; ++m) R.done_col[R.col_first[m]] = (short)m;
  bool touched[NEDOF] = {};
  for (int T = KS_NNZ - 1; T >= 0; --T) {
    const int b = T / 9, c = (T % 9) / 3, d = T % 3, n = BT.n[b], m = BT.m[b];
    R.first_a[T] = !touched[3 * n + c];
    touched[3 * n + c] = true;
    R.first_b[T] = false;
    if (n != m) {
      R.first_b[T] = !touched[3 * m + d];
      touched[3 * m + d] = true;
    }
  }
  return R;
}
constexpr Traversal TR = make_traversal();

// Per-lane state of one group walk.
template <int KR>
struct Walk {
  float p[NEDOF];          // p_e column of this lane (current group)
  float y[NEDOF];          // y_e = K_e p_e, rows formed lazily and stored when complete
  float pn[NEDOF], zn[NEDOF];  // next group's raw p_old and z values
  const int* pos;          // this group's gather positions (shared memory)
  const int* gnext;        // next group's dof numbers (shared memory)
  const float* pold;       // p_old + j
  const float* zsrc;       // z + j (p_old + j for a plain apply)
  float* Y;                // Y + j
  bool valid, nvalid;      // this / the next group's element exists
  bool combine;            // p = z + beta p_old (PCG iteration) or p = p_old (plain apply)
  float beta;
  __device__ __forceinline__ float form(float a, float b) const { return combine ? fmaf(beta, a, b) : a; }
};
constexpr int LAG = 4;     // columns between issuing a node's next-group loads and combining them

// Column at which the next group's values of node K are loaded: node K at
// column K for K <= 21, nodes 22..26 at columns 8..12.  Loading at column
// K alone would hold the most registers just after the walk starts (columns
// 24 and 23); deferring the last five keeps the peak at 144 values (p, y and
// next-group values together) instead of 162.
constexpr int load_column(int K) { return K <= 21 ? K : K - 14; }

template <int KR, int K>
__device__ __forceinline__ void load_next(Walk<KR>& w, int nan) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int gd = w.nvalid ? w.gnext[(3 * K + c) * (1 - nan)] : 0;
    w.pn[3 * K + c] = w.pold[(size_t)gd * KR];
    w.zn[3 * K + c] = w.zsrc[(size_t)gd * KR];
  }
}
template <int KR, int K>
__device__ __forceinline__ void form_next(Walk<KR>& w) {
#pragma unroll
  for (int c = 0; c < 3; ++c) w.pn[3 * K + c] = w.form(w.pn[3 * K + c], w.zn[3 * K + c]);
}

template <int KR, int M>
__device__ __forceinline__ void column_done(Walk<KR>& w) {
  if (w.valid) {
    const int q = w.pos[M];
    if (q >= 0) {
      float* dst = w.Y + (size_t)q * 3 * KR;
      dst[0] = w.y[3 * M];
      dst[KR] = w.y[3 * M + 1];
      dst[2 * KR] = w.y[3 * M + 2];
    }
  }
  // The next group's loads, and the shared-memory reads of their dof
  // numbers, must not be scheduled before this point, where registers have
  // been freed: the index they read depends on a test of the completed row
  // that the compiler cannot decide ahead (y != y only for a NaN, and then
  // the group's first dof number is read instead, a valid one).
  const int nan = w.y[3 * M] != w.y[3 * M];
  if constexpr (M <= 21) load_next<KR, M>(w, nan);
  if constexpr (M >= 8 && M <= 12) load_next<KR, M + 14>(w, nan);
  // loads issued LAG columns ago have had time to land: form p = z + beta
  // p_old for those nodes now, which frees their z registers
  constexpr int MC = M + LAG;
  if constexpr (MC <= 21) form_next<KR, MC>(w);
  if constexpr (MC >= 8 && MC <= 12) form_next<KR, MC + 14>(w);
}

// one stored entry T with value v (walking down)
template <int KR, int T>
__device__ __forceinline__ void entry(float v, Walk<KR>& w) {
  if constexpr (T < KS_NNZ) {
    constexpr int b = T / 9, c = (T % 9) / 3, d = T % 3;
    constexpr int n = BT.n[b], m = BT.m[b];
    if constexpr (TR.first_a[T]) w.y[3 * n + c] = v * w.p[3 * m + d];
    else w.y[3 * n + c] = fmaf(v, w.p[3 * m + d], w.y[3 * n + c]);
    if constexpr (n != m) {
      if constexpr (TR.first_b[T]) w.y[3 * m + d] = v * w.p[3 * n + c];
      else w.y[3 * m + d] = fmaf(v, w.p[3 * n + c], w.y[3 * m + d]);
    }
    if constexpr (TR.done_col[T] >= 0) column_done<KR, TR.done_col[T]>(w);
  }
}

// the float4 pieces of chunk C, last piece first
template <int KR, int C, int NF, int... F>
__device__ __forceinline__ void chunk_entries(const float4* __restrict__ src, Walk<KR>& w,
                                              std::integer_sequence<int, F...>) {
  (
      [&] {
        constexpr int G = NF - 1 - F;
        const float4 v = src[G];
        constexpr int T = (C * CHF) + 4 * G;
        entry<KR, T + 3>(v.w, w);
        entry<KR, T + 2>(v.z, w);
        entry<KR, T + 1>(v.y, w);
        entry<KR, T + 0>(v.x, w);
      }(),
      ...);
}

template <typename F, int... Cs>
__device__ __forceinline__ void for_steps(F& f, std::integer_sequence<int, Cs...>) {
  (f(std::integral_constant<int, Cs>{}), ...);
}

constexpr unsigned chunk_bytes(int c) { return (unsigned)(c == NCH - 1 ? LAST_F4 * 16 : CHF * 4); }

constexpr int IDX = NEDOF + NGLL;  // per element: 81 dof numbers + 27 gather positions
constexpr int NIBUF = 3;           // index buffers per warp: this group, the next, the one after

template <int KR>
struct Shape {
  static constexpr int EPW = 32 / KR;                       // elements per warp
  static constexpr int STAGE_F = EPW * CHF;                 // floats per stage
  static constexpr int RING_F = NSTAGE * STAGE_F;           // floats per warp ring
  static constexpr int GIDX = EPW * IDX;                    // ints per group of indices
  static constexpr int IBUF = NIBUF * GIDX;                 // ints per warp
  static constexpr int BAR_BYTES = 512;                     // NW * NSTAGE mbarriers, padded
  static constexpr size_t SMEM = BAR_BYTES + (size_t)NW * RING_F * 4 + (size_t)NW * IBUF * 4;
};

__device__ __forceinline__ void cp_async4(int* dst, const int* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

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

// Lane 0 issues the chunk at walk position s (chunk NCH-1-s) of group g (all
// of its valid elements) into stage s % NSTAGE; returns false when the group
// is past the end (nothing issued).
template <int KR>
__device__ __forceinline__ bool issue_chunk(const float* __restrict__ Ks, int nelmt, int ngroups, int g, int s,
                                            float* ring, uint64_t* bar) {
  using S = Shape<KR>;
  if (g >= ngroups) return false;
  const int c = NCH - 1 - s;
  const int e0 = g * S::EPW;
  const int nv = min(S::EPW, nelmt - e0);
  const unsigned bytes = chunk_bytes(c);
  float* dst = ring + (s % NSTAGE) * S::STAGE_F;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  expect_tx(bar + (s % NSTAGE), bytes * (unsigned)nv);
  for (int i = 0; i < nv; ++i)
    bulk_copy(dst + i * CHF, Ks + (size_t)(e0 + i) * KS_STRIDE + (size_t)c * CHF, bytes, bar + (s % NSTAGE));
  return true;
}

template <int KR>
__global__ void __launch_bounds__(NW * 32, 1) k_apply_lanes(
    const float* __restrict__ Ks, const int* __restrict__ ge, int nelmt, const float* __restrict__ pold,
    const float* __restrict__ z, int combine, float* __restrict__ Y, const ColState* __restrict__ cs,
    const PcgGlobal* __restrict__ G, const int* __restrict__ pos, int* __restrict__ err) {
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
    for (int st = 0; st < NSTAGE; ++st) mbar_init(bar + st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  Walk<KR> w;
  w.combine = combine != 0;
  w.beta = combine ? (float)cs[j].beta : 0.f;
  w.pold = pold + j;
  w.zsrc = (combine ? z : pold) + j;
  w.Y = Y + j;
  // walk positions issued / waited, counted along the warp's sequence
  int issued = 0, waited = 0;
  if (lane == 0)
    for (int st = 0; st < NSTAGE - 1; ++st) issued += issue_chunk<KR>(Ks, nelmt, ngroups, g, st, ring, bar);
  issued = __shfl_sync(0xffffffffu, issued, 0);
  // indices of this group and the next; the loads of this group's p and z
  // go out once its indices have landed
  prefetch_indices<KR>(ge, pos, nelmt, ngroups, g, ibuf, lane);
  prefetch_indices<KR>(ge, pos, nelmt, ngroups, g + gstride, ibuf + S::GIDX, lane);
  cp_async_wait_1();
  __syncwarp();
  {
    const int* gi = ibuf + i * IDX;
    const bool v0 = g < ngroups && g * S::EPW + i < nelmt;
#pragma unroll
    for (int r = 0; r < NEDOF; ++r) {
      const int gd = v0 ? gi[r] : 0;
      w.pn[r] = w.form(w.pold[(size_t)gd * KR], w.zsrc[(size_t)gd * KR]);
    }
  }
  bool ok = true;
  for (int k = 0; g < ngroups && ok; g += gstride, ++k) {
    const int e = g * S::EPW + i;
    w.valid = e < nelmt;
    w.nvalid = (g + gstride) < ngroups && (g + gstride) * S::EPW + i < nelmt;
#pragma unroll
    for (int r = 0; r < NEDOF; ++r) w.p[r] = w.pn[r];
    // indices two groups ahead go out now; the next group's have landed
    prefetch_indices<KR>(ge, pos, nelmt, ngroups, g + 2 * gstride, ibuf + ((k + 2) % NIBUF) * S::GIDX, lane);
    cp_async_wait_1();
    __syncwarp();
    w.pos = ibuf + (k % NIBUF) * S::GIDX + i * IDX + NEDOF;
    w.gnext = ibuf + ((k + 1) % NIBUF) * S::GIDX + i * IDX;
    const float* mine = ring + i * CHF;
    auto step = [&](auto cc) {
      constexpr int SQ = decltype(cc)::value;   // walk position
      constexpr int C = NCH - 1 - SQ;           // chunk
      if (!ok) return;
      // refill the stage consumed by the previous position: position
      // SQ + NSTAGE - 1 of this group, or of the warp's next group
      if (lane == 0) {
        constexpr int SN = SQ + NSTAGE - 1;
        issued += (SN < NCH) ? issue_chunk<KR>(Ks, nelmt, ngroups, g, SN, ring, bar)
                             : issue_chunk<KR>(Ks, nelmt, ngroups, g + gstride, SN - NCH, ring, bar);
      }
      // the verdict is made warp-uniform so that no lane leaves the
      // shared __syncwarp sequence alone
      const bool wt = __all_sync(0xffffffffu, mbar_wait(bar + (SQ % NSTAGE), (unsigned)((SQ / NSTAGE) & 1)));
      if (!wt) {
        if (lane == 0) atomicExch(err, 1);
        ok = false;
        return;
      }
      ++waited;
      const float4* src = reinterpret_cast<const float4*>(mine + (SQ % NSTAGE) * S::STAGE_F);
      constexpr int NF = (C == NCH - 1) ? LAST_F4 : CHF / 4;
      chunk_entries<KR, C, NF>(src, w, std::make_integer_sequence<int, NF>{});
      __syncwarp();
    };
    for_steps(step, std::make_integer_sequence<int, NCH>{});
    // the nodes whose next-group values were not formed during the walk
    // (load column below LAG: nodes 0 .. LAG-1)
#pragma unroll
    for (int r = 0; r < 3 * LAG; ++r) w.pn[r] = w.form(w.pn[r], w.zn[r]);
    static_assert(load_column(22) - LAG >= 0 && LAG <= 8, "deferred nodes are formed during the walk");
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
                        float* Y, const ColState* cs, const PcgGlobal* G, const int* pos, int* err, cudaStream_t s) {
  using S = lanes::Shape<KR>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(lanes::k_apply_lanes<KR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    attr = true;
  }
  const int ngroups = (nelmt + S::EPW - 1) / S::EPW;
  const int warps = (ngroups + lanes::NW - 1) / lanes::NW;
  int grid = warps < 152 ? warps : 152;
  if (grid < 1) return;
  lanes::k_apply_lanes<KR><<<grid, lanes::NW * 32, S::SMEM, s>>>(Ks, ge, nelmt, pold, z, combine, Y, cs, G, pos, err);
}

size_t apply_lanes_smem(int KR) {
  return KR == 8 ? lanes::Shape<8>::SMEM : KR == 16 ? lanes::Shape<16>::SMEM : lanes::Shape<4>::SMEM;
}

template void launch_apply_lanes<8>(const float*, const int*, int, const float*, const float*, int, float*,
                                    const ColState*, const PcgGlobal*, const int*, int*, cudaStream_t);
template void launch_apply_lanes<16>(const float*, const int*, int, const float*, const float*, int, float*,
                                     const ColState*, const PcgGlobal*, const int*, int*, cudaStream_t);

}  // namespace sg
