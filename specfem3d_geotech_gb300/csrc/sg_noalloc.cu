// sg_noalloc.cu -- sg_pcg_solve_noalloc: the pcg_solver drop-in for callers
// that cannot allocate device memory.
//
// Who needs it: hosts that own the GPU's memory themselves and forbid other
// code from calling cudaMalloc -- for example a Fortran or C++ application
// that runs under a fixed memory pool or a sub-allocator, or a library loaded
// into a process whose allocator must not be bypassed.  sg_pcg_solve needs a context (sg_create),
// and the context allocates; this entry point needs neither.
//
// How: all device memory the solve uses -- the copies of the caller's
// arrays, the PCG vectors, the element products, the block partials and the
// gather topology -- lives in one file-scope static device array of
// SG_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU that loads the library holds
// this array until the process exits.  A call whose arrays do not fit is
// rejected with SG_ERR_BADARG and a message; nothing is allocated.
//
// Set-up: the first call on a device (with that device current) looks up the
// device address of the array with cudaGetSymbolAddress; make that first call
// before any stream capture.  Calls share the array and keep the previous
// call's contents: everything that must start at zero is cleared by each call.
// Calls that overlap on the GPU (several host threads, or several devices'
// work interleaved on one) race on the array and must be serialised by the
// caller.  Work is issued on the legacy default stream and the call returns
// after it completes.
#include <cstring>
#include <string>
#include <vector>

#include "sg_kernels.cuh"

using namespace sg;

namespace {

constexpr size_t SG_NOALLOC_SCRATCH_BYTES = size_t(64) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[SG_NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
// Device address of the scratch array per device, looked up on the first call.
// Written without a lock: two threads making their first call on one device
// at the same time both store the same address, so the race is benign (and
// their solves would race on the array anyway; the caller serialises them).
unsigned char* g_scratch_addr[MAX_DEVICES] = {};

void tag(char* errtag, const std::string& msg) {
  if (!errtag) return;
  size_t n = msg.size() < (size_t)SG_ERRTAG_LEN ? msg.size() : (size_t)SG_ERRTAG_LEN;
  std::memcpy(errtag, msg.data(), n);
  std::memset(errtag + n, ' ', SG_ERRTAG_LEN - n);
}

size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

// Deterministic gather topology built on the device from the element dof map
// (the same groups as the host builder: a node is keyed by its smallest
// non-zero dof; one group per key k = 1..neq, empty groups are skipped).
__global__ void k_topo_count(const int* __restrict__ ge, int nslots, int* __restrict__ key,
                             int* __restrict__ cnt) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const int* g = ge + 3 * (size_t)s;
  int k = 0;
  for (int d = 0; d < 3; ++d)
    if (g[d] > 0 && (k == 0 || g[d] < k)) k = g[d];
  key[s] = k;
  if (k) atomicAdd(cnt + k, 1);
}

// exclusive scan of cnt[0..n) into ptr[0..n], one block, fixed order
__global__ void k_topo_scan(const int* __restrict__ cnt, int n, int* __restrict__ ptr) {
  __shared__ int tot[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int chunk = (n + T - 1) / T;
  const int a = t * chunk, b = min(n, a + chunk);
  int s = 0;
  for (int i = a; i < b; ++i) s += cnt[i];
  tot[t] = s;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int i = 0; i < T; ++i) { int v = tot[i]; tot[i] = run; run += v; }
  }
  __syncthreads();
  int run = tot[t];
  for (int i = a; i < b; ++i) { ptr[i] = run; run += cnt[i]; }
  if (b == n && a < b) ptr[n] = run;
  if (n == 0 && t == 0) ptr[0] = 0;
}

__global__ void k_topo_fill(const int* __restrict__ ge, const int* __restrict__ key, int nslots,
                            const int* __restrict__ ptr, int* __restrict__ fillc, int* __restrict__ ent,
                            int* __restrict__ dof) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  int k = key[s];
  if (!k) return;
  int pos = ptr[k] + atomicAdd(fillc + k, 1);
  ent[pos] = s;
  // every slot of a node carries the same three dof numbers
  for (int d = 0; d < 3; ++d) dof[3 * (size_t)k + d] = ge[3 * (size_t)s + d];
}

// groups are the keys that occur, numbered in increasing key order (the host
// builder's numbering): flag the occupied keys ...
__global__ void k_topo_flags(const int* __restrict__ cnt, int n, int* __restrict__ flag) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) flag[k] = (k >= 1 && cnt[k] > 0) ? 1 : 0;
}

// ... and move each occupied key's range and dof triple to its group index
__global__ void k_topo_compact(const int* __restrict__ flag, const int* __restrict__ gid,
                               const int* __restrict__ ptr, const int* __restrict__ dof, int n,
                               int* __restrict__ gptr, int* __restrict__ gdof) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && flag[k]) {
    int g = gid[k];
    gptr[g] = ptr[k];
    for (int d = 0; d < 3; ++d) gdof[3 * (size_t)g + d] = dof[3 * (size_t)k + d];
  }
  if (k == 0) gptr[gid[n]] = ptr[n];
}

// gather position of every slot (its index in ent), -1 for slots of fully fixed nodes
__global__ void k_topo_pos(const int* __restrict__ ent, int nent, int* __restrict__ pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nent) pos[ent[i]] = i;
}

// restore increasing element order inside each group (insertion sort)
__global__ void k_topo_sort(const int* __restrict__ ptr, int n, int* __restrict__ ent) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  for (int i = ptr[k] + 1; i < ptr[k + 1]; ++i) {
    int v = ent[i], j = i - 1;
    while (j >= ptr[k] && ent[j] > v) { ent[j + 1] = ent[j]; --j; }
    ent[j + 1] = v;
  }
}

}  // namespace

extern "C" int sg_pcg_solve_noalloc(int neq, int nelmt, int nedof, const double* k, double* u, const double* f,
                                    const double* dprecon, const int* gdof_elmt, int cg_maxiter, double cg_tol,
                                    int* cg_iter, char* errtag) {
  tag(errtag, "ERROR: unknown!");
  if (nedof != NEDOF || neq < 0 || nelmt < 0 || !k || !u || !f || !dprecon || !gdof_elmt || !cg_iter) {
    tag(errtag, "ERROR: bad argument to sg_pcg_solve_noalloc (nedof must be 81)!");
    return SG_ERR_BADARG;
  }
  for (size_t i = 0; i < (size_t)nelmt * NEDOF; ++i)
    if (gdof_elmt[i] < 0 || gdof_elmt[i] > neq) {
      tag(errtag, "ERROR: gdof_elmt entry out of [0,neq]!");
      return SG_ERR_BADARG;
    }
  const size_t n1 = (size_t)neq + 1, nslots = (size_t)nelmt * NGLL;
  {
    // The device builds one gather group per node, keyed by the node's
    // smallest free dof, and takes the group's dof triple from any of its
    // slots.  A dof map in which two slots share that key but not all three
    // dofs is not a node numbering; reject it so that this call gives the same
    // solve as sg_pcg_solve (host memory only).
    std::vector<int> trip(3 * n1, -1);
    for (size_t sl = 0; sl < nslots; ++sl) {
      const int* g = gdof_elmt + 3 * sl;
      int key = 0;
      for (int d = 0; d < 3; ++d)
        if (g[d] > 0 && (key == 0 || g[d] < key)) key = g[d];
      if (!key) continue;
      int* t = trip.data() + 3 * (size_t)key;
      if (t[0] < 0) {
        t[0] = g[0]; t[1] = g[1]; t[2] = g[2];
      } else if (t[0] != g[0] || t[1] != g[1] || t[2] != g[2]) {
        tag(errtag, "ERROR: gdof_elmt gives one dof to nodes with different dof triples!");
        return SG_ERR_BADARG;
      }
    }
  }
  // scratch layout
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += up256(bytes); return o; };
  const size_t oK = take(sizeof(double) * (size_t)nelmt * NEDOF * NEDOF);
  const size_t oGe = take(sizeof(int) * (size_t)nelmt * NEDOF);
  const size_t oU = take(sizeof(double) * n1), oF = take(sizeof(double) * n1), oD = take(sizeof(double) * n1);
  const size_t oR = take(sizeof(double) * n1), oZ = take(sizeof(double) * n1), oP = take(sizeof(double) * n1);
  const size_t oKp = take(sizeof(double) * n1);
  const size_t oY = take(sizeof(double) * (size_t)nelmt * NEDOF);
  const size_t oPart = take(sizeof(double) * NPART * 16 * 4);
  const size_t oCs = take(sizeof(ColState) * 16), oG = take(sizeof(PcgGlobal));
  const size_t oKey = take(sizeof(int) * nslots), oEnt = take(sizeof(int) * nslots);
  const size_t oCnt = take(sizeof(int) * (n1 + 1)), oPtr = take(sizeof(int) * (n1 + 1));
  const size_t oFill = take(sizeof(int) * (n1 + 1)), oDof = take(sizeof(int) * 3 * (n1 + 1));
  const size_t oFlag = take(sizeof(int) * (n1 + 1)), oGid = take(sizeof(int) * (n1 + 1));
  const size_t oGptr = take(sizeof(int) * (n1 + 1)), oGdof = take(sizeof(int) * 3 * (n1 + 1));
  const size_t oPos = take(sizeof(int) * nslots);
  if (off > SG_NOALLOC_SCRATCH_BYTES) {
    tag(errtag, "ERROR: problem needs " + std::to_string(off >> 20) +
                    " MiB of device scratch; sg_pcg_solve_noalloc is limited to 64 MiB (use sg_pcg_solve)!");
    return SG_ERR_BADARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    tag(errtag, "ERROR: no usable CUDA device!");
    return SG_ERR_NODEVICE;
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      tag(errtag, std::string("ERROR: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return SG_ERR_CUDA;
    }
    g_scratch_addr[dev] = (unsigned char*)p;
  }
  unsigned char* base = g_scratch_addr[dev];
  double* dK = (double*)(base + oK);
  int* dGe = (int*)(base + oGe);
  double *dU = (double*)(base + oU), *dF = (double*)(base + oF), *dDp = (double*)(base + oD);
  double *dR = (double*)(base + oR), *dZ = (double*)(base + oZ), *dP = (double*)(base + oP);
  double* dKp = (double*)(base + oKp);
  double* dY = (double*)(base + oY);
  double* dPart = (double*)(base + oPart);
  ColState* dCs = (ColState*)(base + oCs);
  PcgGlobal* dG = (PcgGlobal*)(base + oG);
  int *dKey = (int*)(base + oKey), *dEnt = (int*)(base + oEnt), *dCnt = (int*)(base + oCnt);
  int *dPtr = (int*)(base + oPtr), *dFill = (int*)(base + oFill), *dDof = (int*)(base + oDof);
  int *dFlag = (int*)(base + oFlag), *dGid = (int*)(base + oGid), *dGptr = (int*)(base + oGptr);
  int* dGdof = (int*)(base + oGdof);
  int* dPos = (int*)(base + oPos);
  cudaStream_t s = 0;
  cudaMemcpyAsync(dK, k, sizeof(double) * (size_t)nelmt * NEDOF * NEDOF, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dGe, gdof_elmt, sizeof(int) * (size_t)nelmt * NEDOF, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dU, u, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dF, f, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dDp, dprecon, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  // topology: counters and the dof table start at zero on every call
  cudaMemsetAsync(dCnt, 0, sizeof(int) * (n1 + 1), s);
  cudaMemsetAsync(dFill, 0, sizeof(int) * (n1 + 1), s);
  cudaMemsetAsync(dDof, 0, sizeof(int) * 3 * (n1 + 1), s);
  if (nslots) {
    k_topo_count<<<(unsigned)((nslots + 255) / 256), 256, 0, s>>>(dGe, (int)nslots, dKey, dCnt);
  }
  k_topo_scan<<<1, 1024, 0, s>>>(dCnt, (int)n1, dPtr);
  if (nslots) {
    k_topo_fill<<<(unsigned)((nslots + 255) / 256), 256, 0, s>>>(dGe, dKey, (int)nslots, dPtr, dFill, dEnt, dDof);
  }
  k_topo_sort<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(dPtr, (int)n1, dEnt);
  k_topo_flags<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(dCnt, (int)n1, dFlag);
  k_topo_scan<<<1, 1024, 0, s>>>(dFlag, (int)n1, dGid);
  k_topo_compact<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(dFlag, dGid, dPtr, dDof, (int)n1, dGptr, dGdof);
  cudaMemsetAsync(dPos, 0xff, sizeof(int) * nslots, s);  // -1 everywhere, then the occupied slots
  int nent = 0;
  cudaMemcpy(&nent, dPtr + n1, sizeof(int), cudaMemcpyDeviceToHost);
  if (nent > 0) k_topo_pos<<<(unsigned)((nent + 255) / 256), 256, 0, s>>>(dEnt, nent, dPos);
  int ngroups = 0;
  if (cudaMemcpy(&ngroups, dGid + n1, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    tag(errtag, std::string("ERROR: CUDA failure: ") + cudaGetErrorString(cudaGetLastError()));
    return SG_ERR_CUDA;
  }
  // the same groups, in the same order, as the host builder used by sg_pcg_solve
  GatherTopo T;
  T.ngroups = ngroups;
  T.d_ptr = dGptr;
  T.d_ent = dEnt;
  T.d_dof = dGdof;
  T.d_pos = dPos;
  // PCG state: per-column scalars, control word, direction and product start at zero
  ColState hcs[16];
  std::memset(hcs, 0, sizeof(hcs));
  hcs[0].tol = cg_tol;
  hcs[0].active = 1;
  PcgGlobal hg;
  std::memset(&hg, 0, sizeof(hg));
  hg.maxiter = cg_maxiter;
  hg.kcols = 1;
  cudaMemcpyAsync(dCs, hcs, sizeof(hcs), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dG, &hg, sizeof(hg), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dP, 0, sizeof(double) * n1, s);
  cudaMemsetAsync(dKp, 0, sizeof(double) * n1, s);
  // kp = K u, r = f - kp, z = D r, p = z (src/solver.f90:38-50)
  pcg_apply<double, 1>(1, dK, dGe, nelmt, dU, (const double*)nullptr, 0, dY, dCs, dG, nullptr, dPos, &dG->err, s);
  pcg_gather<double, 1>(T, dY, dKp, dP, dZ, 0, dCs, dG, dPart, s);
  pcg_update<double, 1>((int)n1, dU, dR, dZ, dP, dKp, dF, dDp, 1, dCs, dG, dPart, s);
  const int chunk = 16;
  int status = SG_OK;
  PcgGlobal got;
  for (;;) {
    for (int c = 0; c < chunk; ++c) {
      pcg_apply<double, 1>(1, dK, dGe, nelmt, dP, dZ, 1, dY, dCs, dG, nullptr, dPos, &dG->err, s);
      pcg_gather<double, 1>(T, dY, dKp, dP, dZ, 1, dCs, dG, dPart, s);
      pcg_update<double, 1>((int)n1, dU, dR, dZ, dP, dKp, dF, dDp, 0, dCs, dG, dPart, s);
    }
    if (cudaMemcpy(&got, dG, sizeof(got), cudaMemcpyDeviceToHost) != cudaSuccess) {
      status = SG_ERR_CUDA;
      break;
    }
    if (got.all_done) break;
    if (got.it >= cg_maxiter + chunk) { status = SG_ERR_TIMEOUT; break; }
  }
  ColState res;
  cudaError_t e1 = cudaMemcpy(&res, dCs, sizeof(res), cudaMemcpyDeviceToHost);
  cudaError_t e2 = cudaMemcpy(u, dU, sizeof(double) * n1, cudaMemcpyDeviceToHost);
  if (status == SG_ERR_CUDA || e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaError_t e = cudaGetLastError();
    tag(errtag, std::string("ERROR: CUDA failure: ") + cudaGetErrorString(e));
    return SG_ERR_CUDA;
  }
  *cg_iter = res.iters;
  if (status == SG_ERR_TIMEOUT) {
    tag(errtag, "ERROR: PCG iteration guard reached!");
    return SG_ERR_TIMEOUT;
  }
  if (res.failed) {
    tag(errtag, "ERROR: PCG solver doesn't converge!");
    return SG_ERR_NOCONV;
  }
  tag(errtag, "");
  return SG_OK;
}
