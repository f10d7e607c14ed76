// sg_apply_tc.cu -- batched element apply on the 5th-generation tensor cores.
//
// For k = 8 or 16 concurrent SRF trials the element apply is a small dense
// contraction per element, Y_e[81 x k] = K_e[81 x 81] P_e[81 x k], which runs
// here as one tcgen05.mma chain per element:
//   D[128 x 16] (TMEM, FP32) = A[128 x 96] B[96 x 16],  kind::tf32,
// with A = K_e (rows and columns beyond 81 are padding) and B^T = P_e^T
// (columns beyond k are zero).  FP32 accuracy comes from the 3xTF32 split
// x = hi + lo (hi = x rounded to TF32, lo = x - hi): D = Ahi Bhi + Ahi Blo + Alo Bhi.
//
// Per CTA (one warpgroup, one CTA per SM) the element loop is double-buffered:
//   - thread 0 streams the next element's sparse symmetric K_e (9.7 KB) into
//     shared memory with cp.async.bulk (TMA), completion on an mbarrier;
//   - all 128 threads expand the stored 3x3 node blocks into the two
//     128B-swizzled K-major A tiles (hi, lo) and gather, combine and split
//     P_e into the B tiles;
//   - thread 0 issues the 36 MMAs of the element into one of two TMEM
//     accumulators and commits them to an mbarrier;
//   - meanwhile the warpgroup drains the previous element's accumulator with
//     tcgen05.ld and writes its rows to the gather positions.
// Every mbarrier wait is bounded; a timeout records the fault in a device flag
// and the CTA drains its outstanding copies and MMAs (bounded) before it frees
// TMEM and returns.
#include <cstdint>
#include <cstdio>

#include "sg_kernels.cuh"

namespace sg {

namespace tc {

constexpr int THREADS = 128;
constexpr int N = 16;                 // MMA N (k padded to 16)
constexpr int KPAD = 96;              // K padded to 3 swizzle atoms of 32 TF32
constexpr int A_ATOM = 11 * 1024;     // 11 row groups of 8 rows (88 >= 81 rows) per K atom
constexpr int A_TILE = 3 * A_ATOM;    // 33792 B; the MMA reads 16 row groups and overhangs
                                      // into the following tile -- those rows (88..127) are
                                      // padding whose D rows are never read
constexpr int B_ATOM = 2 * 1024;      // 16 rows = 2 row groups per K atom
constexpr int B_TILE = 3 * B_ATOM;    // 6144 B
constexpr int OFF_A = 0;                               // [stage][hi/lo]
constexpr int OFF_B = OFF_A + 4 * A_TILE;             // 135168
constexpr int OFF_K = OFF_B + 4 * B_TILE;             // 159744, sparse K staging [stage]
constexpr int KBYTES = KS_STRIDE * 4;                  // 9728
constexpr int OFF_ENT = OFF_K + 2 * KBYTES;           // 179200, entry table
constexpr int OFF_BAR = OFF_ENT + ((KS_NNZ * 4 + 127) / 128) * 128;
constexpr int SMEM_BYTES = OFF_BAR + 128 + 1024;       // + alignment slack
constexpr uint32_t TMEM_COLS = 32;                     // two 16-column accumulators

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((128u >> 4) << 24);


// KR consecutive floats with 16-byte loads
template <int KR>
__device__ __forceinline__ void load_row(const float* __restrict__ src, float (&out)[KR]) {
#pragma unroll
  for (int q = 0; q < KR / 4; ++q) {
    float4 t = reinterpret_cast<const float4*>(src)[q];
    out[4 * q] = t.x; out[4 * q + 1] = t.y; out[4 * q + 2] = t.z; out[4 * q + 3] = t.w;
  }
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset
// 16 B (unused by swizzled K-major), stride byte offset 1024 B between 8-row
// groups (bits 32-45), version 1 (bit 46), 128-byte swizzle (bits 61-63 = 2).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// byte offset of element (row, k) in a 128B-swizzled K-major tile whose K
// atoms (32 FP32 each) are atom_bytes apart
__device__ __forceinline__ uint32_t swz(int row, int k, int atom_bytes) {
  const int a = k >> 5, kk = k & 31;
  const int r8 = row & 7;
  return (uint32_t)(a * atom_bytes + (row >> 3) * 1024 + r8 * 128 + ((((kk >> 2) ^ r8)) << 4) + ((kk & 3) << 2));
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int tries = 0; tries < (1 << 22); ++tries) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
      "l"(src), "r"(bytes), "r"(saddr(bar))
      : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int KR>
__global__ void __launch_bounds__(THREADS, 1) k_apply_tc(const float* __restrict__ Ks, const int* __restrict__ ge,
                                                          int nelmt, const float* __restrict__ pold,
                                                          const float* __restrict__ z, int combine, float* __restrict__ Y,
                                                          const ColState* __restrict__ cs, const PcgGlobal* __restrict__ G,
                                                          const int* __restrict__ entry_g, const int* __restrict__ pos,
                                                          int* __restrict__ err) {
  if (G && G->all_done) return;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned working base (the 128B swizzle pattern uses address bits 7-9)
  unsigned char* sm = smem_raw + ((1024 - (saddr(smem_raw) & 1023)) & 1023);
  int* ent = (int*)(sm + OFF_ENT);
  uint64_t* kbar = (uint64_t*)(sm + OFF_BAR);
  uint64_t* mbar = kbar + 2;
  uint32_t* tmem_slot = (uint32_t*)(kbar + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // zero the A and B tiles once: padding rows/columns and the structural
  // zeros of K_e are never written again
  for (int i = tid; i < (OFF_K - OFF_A) / 16; i += THREADS) reinterpret_cast<float4*>(sm + OFF_A)[i] = make_float4(0, 0, 0, 0);
  for (int i = tid; i < KS_NNZ; i += THREADS) ent[i] = entry_g[i];
  if (tid == 0) {
    mbar_init(&kbar[0], 1); mbar_init(&kbar[1], 1);
    mbar_init(&mbar[0], 1); mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  float beta[KR];
#pragma unroll
  for (int j = 0; j < KR; ++j) beta[j] = combine ? (float)cs[j].beta : 0.f;
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  const int stride = gridDim.x;
  int e = blockIdx.x;
  int issued = 0, kwaited = 0, committed = 0, mwaited = 0;
  bool fault = false;
  if (e < nelmt && tid == 0) {
    bulk_load(sm + OFF_K, Ks + (size_t)e * KS_STRIDE, KBYTES, &kbar[0]);
    issued = 1;
  }
  int eprev = -1, niter = 0;
  for (int i = 0; e < nelmt; ++i, e += stride) {
    niter = i + 1;
    const int s = i & 1;
    const int en = e + stride;
    if (tid == 0 && en < nelmt) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_load(sm + OFF_K + (s ^ 1) * KBYTES, Ks + (size_t)en * KS_STRIDE, KBYTES, &kbar[s ^ 1]);
      ++issued;
    }
    // B tile: P_e (combined) -> hi/lo, row j = RHS column, k = element dof 3a+d
    unsigned char* Bh = sm + OFF_B + (s * 2 + 0) * B_TILE;
    unsigned char* Bl = sm + OFF_B + (s * 2 + 1) * B_TILE;
    if (tid < NEDOF) {
      const int g = ge[(size_t)e * NEDOF + tid];
      float pv[KR];
      load_row<KR>(pold + (size_t)g * KR, pv);
      if (combine) {
        float zv[KR];
        load_row<KR>(z + (size_t)g * KR, zv);
#pragma unroll
        for (int j = 0; j < KR; ++j) pv[j] = fmaf(beta[j], pv[j], zv[j]);
      }
#pragma unroll
      for (int j = 0; j < KR; ++j) {
        float h = tf32_hi(pv[j]);
        const uint32_t o = swz(j, tid, B_ATOM);
        *(float*)(Bh + o) = h;
        *(float*)(Bl + o) = pv[j] - h;
      }
    }
    // wait for this element's K_e, expand into the A tiles
    bool ok = mbar_wait(&kbar[s], (unsigned)((i >> 1) & 1));
    ++kwaited;
    if (!ok) { fault = true; }
    if (!fault) {
      const float* kst = (const float*)(sm + OFF_K + s * KBYTES);
      unsigned char* Ah = sm + OFF_A + (s * 2 + 0) * A_TILE;
      unsigned char* Al = sm + OFF_A + (s * 2 + 1) * A_TILE;
      for (int t = tid; t < KS_NNZ; t += THREADS) {
        const int pk = ent[t];
        const int row = pk & 255, col = pk >> 8;
        const float v = kst[t];
        const float h = tf32_hi(v), l = v - h;
        uint32_t o = swz(row, col, A_ATOM);
        *(float*)(Ah + o) = h;
        *(float*)(Al + o) = l;
        if (row / 3 != col / 3) {  // the transposed copy of a coupled block
          o = swz(col, row, A_ATOM);
          *(float*)(Ah + o) = h;
          *(float*)(Al + o) = l;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    if (__syncthreads_or(fault ? 1 : 0)) { fault = true; break; }
    if (tid == 0) {
      const uint32_t d = tmem + (uint32_t)(s * N);
      const uint32_t abase = saddr(sm + OFF_A + (s * 2) * A_TILE), bbase = saddr(sm + OFF_B + (s * 2) * B_TILE);
      int first = 1;
#pragma unroll 1
      for (int prod = 0; prod < 3; ++prod) {
        const uint32_t ab = abase + (prod == 2 ? A_TILE : 0);   // Alo only in the third product
        const uint32_t bb = bbase + (prod == 1 ? B_TILE : 0);   // Blo only in the second
#pragma unroll
        for (int ks = 0; ks < KPAD / 8; ++ks) {
          const uint32_t koff = (uint32_t)((ks & 3) * 32);   // 8 TF32 = 32 bytes inside the 128-byte atom
          const uint64_t ad = sdesc(ab + (ks >> 2) * A_ATOM + koff);
          const uint64_t bd = sdesc(bb + (ks >> 2) * B_ATOM + koff);
          mma_tf32(d, ad, bd, IDESC, first ? 0 : 1);
          first = 0;
        }
      }
      mma_commit(&mbar[s]);
      ++committed;
    }
    // epilogue of the previous element while this element's MMAs run
    if (eprev >= 0) {
      const int sp = s ^ 1;
      bool okm = mbar_wait(&mbar[sp], (unsigned)(((i - 1) >> 1) & 1));
      ++mwaited;
      if (!okm) fault = true;
      fence_after();
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(sp * N), v);
      const int r = warp * 32 + lane;
      if (!fault && r < NEDOF) {
        const int q = pos[(size_t)eprev * NGLL + r / 3];
        if (q >= 0) {
          float4* yo = reinterpret_cast<float4*>(Y + ((size_t)q * 3 + r % 3) * KR);
#pragma unroll
          for (int j = 0; j < KR / 4; ++j) yo[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
      }
    }
    fence_before();
    __syncthreads();
    fence_after();
    eprev = e;
  }
  // last element
  if (!fault && eprev >= 0) {
    const int last = niter - 1;
    const int sp = last & 1;
    bool okm = mbar_wait(&mbar[sp], (unsigned)((last >> 1) & 1));
    ++mwaited;
    if (!okm) fault = true;
    fence_after();
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(sp * N), v);
    const int r = warp * 32 + lane;
    if (!fault && r < NEDOF) {
      const int q = pos[(size_t)eprev * NGLL + r / 3];
      if (q >= 0) {
        float4* yo = reinterpret_cast<float4*>(Y + ((size_t)q * 3 + r % 3) * KR);
#pragma unroll
        for (int j = 0; j < KR / 4; ++j) yo[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      }
    }
  }
  if (fault && tid == 0) atomicExch(err, 1);
  // drain what is still in flight (bounded), then free TMEM
  if (tid == 0) {
    for (int i = kwaited; i < issued; ++i) mbar_wait(&kbar[i & 1], (unsigned)((i >> 1) & 1));
    for (int i = mwaited; i < committed; ++i) mbar_wait(&mbar[i & 1], (unsigned)((i >> 1) & 1));
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

}  // namespace tc

template <int KR>
void launch_apply_tc(const float* Ks, const int* ge, int nelmt, const float* pold, const float* z, int combine,
                     float* Y, const ColState* cs, const PcgGlobal* G, const int* d_entry, const int* pos,
                     int* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(tc::k_apply_tc<KR>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
    attr = true;
  }
  int grid = nelmt < 152 ? nelmt : 152;
  if (grid < 1) return;
  tc::k_apply_tc<KR><<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(Ks, ge, nelmt, pold, z, combine, Y, cs, G, d_entry,
                                                               pos, err);
}

template void launch_apply_tc<8>(const float*, const int*, int, const float*, const float*, int, float*,
                                 const ColState*, const PcgGlobal*, const int*, const int*, int*, cudaStream_t);
template void launch_apply_tc<16>(const float*, const int*, int, const float*, const float*, int, float*,
                                  const ColState*, const PcgGlobal*, const int*, const int*, int*, cudaStream_t);

}  // namespace sg
