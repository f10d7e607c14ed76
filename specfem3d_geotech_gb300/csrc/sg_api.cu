// sg_api.cu -- C ABI of the solve path (include/sg_solver.h): contexts and
// device memory, the pcg_solver drop-in, the device-resident model, the
// slope3d trial / sweep / factor-of-safety drivers and excavation3d.
//
// Host code here only orchestrates: every vector operation, reduction and
// element computation of the solve runs in the kernels of sg_kernels.cu.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "sg_kernels.cuh"

using namespace sg;

namespace {

constexpr double PI_D = 3.141592653589793;
constexpr double DEG2RAD = PI_D / 180.0, RAD2DEG = 180.0 / PI_D;
constexpr double INFTOL = 1.0e32, ZEROTOL = 1.0e-12;
int g_create_status = SG_OK;

void set_tag(char* errtag, const std::string& msg) {
  if (!errtag) return;
  size_t n = std::min(msg.size(), (size_t)SG_ERRTAG_LEN);
  std::memcpy(errtag, msg.data(), n);
  std::memset(errtag + n, ' ', SG_ERRTAG_LEN - n);  // Fortran blank padding
}

int next_pow2(int k) {
  int r = 1;
  while (r < k) r <<= 1;
  return r;
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct sg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t budget = 0, used = 0;
  std::unordered_map<void*, size_t> live;
  std::string err;
  Profile prof;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  std::vector<std::pair<int, int>> ev_used;  // (pool index, category)
  double* pin = nullptr;                     // pinned scratch for scalars
  int* d_err = nullptr;  // bounded-wait error word of this context's applies outside a PCG solve
  cudaEvent_t marks[16] = {};
  long long launch0 = 0;
  int* d_nbr = nullptr;
  int* d_entry = nullptr;
  // drop-in cache: the reference calls pcg_solver with the same dof map every
  // plastic iteration, so the gather topology is rebuilt only when it changes.
  struct DropIn {
    std::vector<int> ge;
    int neq = -1, nelmt = -1;
    GatherTopo T;
    int* d_ge = nullptr;
    double* d_K = nullptr;
    size_t kcap = 0;
    double *u = nullptr, *f = nullptr, *dp = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *kp = nullptr,
           *Y = nullptr, *part = nullptr;
    int n1cap = 0, necap = 0;
    ColState* cs = nullptr;
    PcgGlobal* G = nullptr;
  } dropin;
  // stress-block drop-in cache: mesh, dof map and element list of the last
  // call (host copies for the content test) and their device forms
  struct StressDropIn {
    std::vector<double> coord;
    std::vector<int> gnum, ge, mat, elist;
    int nnode = -1, nelmt = -1, neq = -1, nel = -1;
    GatherTopo T;  // groups of the listed elements' dof map
    double *d_coord = nullptr, *d_geo = nullptr, *x = nullptr, *evpt = nullptr, *stress = nullptr, *bl = nullptr,
           *Yb = nullptr, *wp = nullptr, *vm = nullptr, *sf = nullptr, *part = nullptr, *red = nullptr;
    int *d_gnum = nullptr, *d_ge = nullptr, *d_mat = nullptr, *d_elist = nullptr;
    MatF* mf = nullptr;
    int mfcap = 0;
  } sdrop;

  // CUDA graphs of PCG iteration chunks on small meshes, where launching
  // three short kernels per iteration from the host costs as much as running
  // them.  Keyed by every argument of the captured launches; a chunk replays
  // exactly the kernels (and arguments) the eager loop would launch.
  struct ChunkGraph {
    std::array<uintptr_t, 26> key{};
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<ChunkGraph> graphs;
  bool graphs_ok = true;
  cudaGraphExec_t chunk_graph(const std::array<uintptr_t, 26>& key, const std::function<void()>& launch) {
    for (auto& g : graphs)
      if (g.key == key) return g.exec;
    if (!graphs_ok) return nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      graphs_ok = false;
      return nullptr;
    }
    launch();
    const cudaError_t e1 = cudaStreamEndCapture(stream, &graph);
    const cudaError_t e2 = (e1 == cudaSuccess) ? cudaGraphInstantiate(&exec, graph, 0) : e1;
    if (graph) cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) {
      cudaGetLastError();
      graphs_ok = false;  // eager launches from now on
      return nullptr;
    }
    if (graphs.size() >= 16) {
      cudaGraphExecDestroy(graphs.front().exec);
      graphs.erase(graphs.begin());
    }
    graphs.push_back({key, exec});
    return exec;
  }
  void drop_graphs() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
    graphs.clear();
  }

  bool check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
  }
  template <typename T>
  T* alloc(size_t n) {
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (budget && used + bytes > budget) { err = "HBM budget exceeded"; return nullptr; }
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) { cudaGetLastError(); err = "cudaMalloc failed"; return nullptr; }
    used += bytes;
    live[p] = bytes;
    return (T*)p;
  }
  void release(void* p) {
    if (!p) return;
    auto it = live.find(p);
    if (it == live.end()) return;  // not ours or already released
    used -= it->second;
    live.erase(it);
    cudaFree(p);
  }
  // profiling: events bracket the launches of one category
  int prof_begin() {
    if (!prof.on) return -1;
    size_t idx = ev_used.size();
    if (idx >= ev_pool.size()) {
      cudaEvent_t a, b;
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      ev_pool.push_back({a, b});
    }
    cudaEventRecord(ev_pool[idx].first, stream);
    return (int)idx;
  }
  void prof_end(int idx, int cat) {
    if (idx < 0) return;
    cudaEventRecord(ev_pool[idx].second, stream);
    ev_used.push_back({idx, cat});
    prof.counts[1]++;
    if (cat == 1) prof.counts[0]++;
    if (ev_used.size() > 4000) prof_flush();
  }
  void prof_flush() {
    if (ev_used.empty()) return;
    cudaStreamSynchronize(stream);
    for (auto& u : ev_used) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev_pool[u.first].first, ev_pool[u.first].second);
      prof.ms[u.second] += ms;
    }
    ev_used.clear();
  }
};

// ---------------------------------------------------------------------------
// PCG driver: kp = K u, r = f - kp, z = D r, p = z, then chunks of fused
// iterations (apply with on-the-fly direction, gather + alpha, update + stop
// test) until every active column stops.  Between chunks the host reads the
// device control word; iterations after a column stops are skipped on device.
// ---------------------------------------------------------------------------
struct Op {
  int dense = 0;
  const void* K = nullptr;
  const int* ge = nullptr;
  int nelmt = 0;
  const GatherTopo* T = nullptr;
};

template <typename V>
struct PcgBufs {
  V *r = nullptr, *z = nullptr, *p = nullptr, *kp = nullptr, *Y = nullptr;
  double* part = nullptr;
  ColState* cs = nullptr;
  PcgGlobal* G = nullptr;
};

template <typename V, int KR>
static int pcg_run_t(sg_ctx* C, const Op& op, const PcgBufs<V>& B, int n1, V* u, const V* f, const V* dp, int kcols,
                     const int* active, int maxiter, double tol, int mode, int* iters, int* failed, int* used_iters,
                     double* laststep = nullptr) {
  cudaStream_t s = C->stream;
  ColState hcs[16];
  std::memset(hcs, 0, sizeof(hcs));
  for (int j = 0; j < KR; ++j) {
    hcs[j].tol = tol;
    hcs[j].active = (j < kcols && active[j]) ? 1 : 0;
  }
  PcgGlobal hg;
  std::memset(&hg, 0, sizeof(hg));
  hg.maxiter = maxiter;
  hg.mode = mode & 3;
  hg.kcols = kcols;
  const bool keep_dir = (mode & 2) != 0;
  if (keep_dir) {
    // continue from the device-resident column state of the previous solve:
    // only the activity mask and tolerances change
    ColState prev[16];
    cudaMemcpyAsync(prev, B.cs, sizeof(ColState) * KR, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int j = 0; j < KR; ++j) {
      prev[j].tol = hcs[j].tol;
      prev[j].active = hcs[j].active;
      hcs[j] = prev[j];
    }
  }
  cudaMemcpyAsync(B.cs, hcs, sizeof(ColState) * KR, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(B.G, &hg, sizeof(hg), cudaMemcpyHostToDevice, s);
  if (!keep_dir) cudaMemsetAsync(B.p, 0, sizeof(V) * (size_t)n1 * KR, s);
  cudaMemsetAsync(B.kp, 0, sizeof(V) * (size_t)n1 * KR, s);
  int ev;
  if (!(mode & 4)) {  // bit 2: the caller guarantees u = 0, so kp = K u = 0 without an apply
    ev = C->prof_begin();
    pcg_apply<V, KR>(op.dense, op.K, op.ge, op.nelmt, u, (const V*)nullptr, 0, B.Y, B.cs, B.G, C->d_nbr, op.T->d_pos,
                     &B.G->err, s);
    C->prof_end(ev, 1);
    pcg_gather<V, KR>(*op.T, B.Y, B.kp, B.p, B.z, 0, B.cs, B.G, B.part, s);
  }
  ev = C->prof_begin();
  pcg_update<V, KR>(n1, u, B.r, B.z, B.p, B.kp, f, dp, 1, B.cs, B.G, B.part, s);
  C->prof_end(ev, 3);
  const int chunk = op.nelmt >= 50000 ? 4 : (op.nelmt >= 5000 ? 16 : 64);
  const auto t0 = std::chrono::steady_clock::now();
  int it = 0;
  int status = SG_OK;
  volatile PcgGlobal* hG = (volatile PcgGlobal*)C->pin;
  // FP32, 8 or 16 columns, stored matrices applied by k_apply_lanes, residual
  // test: two kernels per iteration (the apply forms the direction from the
  // previous step's r and kp; k_pcg_gather_update does the rest)
  bool fused = false;
  if constexpr (std::is_same<V, float>::value && (KR == 8 || KR == 16))
    fused = (mode & 1) && apply_uses_lanes(op.dense, KR) && fused_pcg_enabled();
  auto eager_chunk = [&]() {
    if constexpr (std::is_same<V, float>::value && (KR == 8 || KR == 16)) {
      if (fused) {
        for (int c = 0; c < chunk; ++c) {
          ev = C->prof_begin();
          launch_apply_lanes<KR>((const float*)op.K, op.ge, op.nelmt, B.p, nullptr, 2, B.Y, B.cs, B.G, op.T->d_pos,
                                 &B.G->err, s, FusedDir{B.r, B.kp, dp});
          add_launches(1);
          C->prof_end(ev, 1);
          ev = C->prof_begin();
          pcg_gather_update<KR>(*op.T, B.Y, B.kp, B.p, B.r, u, dp, B.cs, B.G, B.part, s);
          C->prof_end(ev, 2);
        }
        return;
      }
    }
    for (int c = 0; c < chunk; ++c) {
      ev = C->prof_begin();
      pcg_apply<V, KR>(op.dense, op.K, op.ge, op.nelmt, B.p, B.z, 1, B.Y, B.cs, B.G, C->d_nbr, op.T->d_pos,
                       &B.G->err, s);
      C->prof_end(ev, 1);
      ev = C->prof_begin();
      pcg_gather<V, KR>(*op.T, B.Y, B.kp, B.p, B.z, 1, B.cs, B.G, B.part, s);
      C->prof_end(ev, 2);
      ev = C->prof_begin();
      pcg_update<V, KR>(n1, u, B.r, B.z, B.p, B.kp, f, dp, 0, B.cs, B.G, B.part, s);
      C->prof_end(ev, 3);
    }
  };
  // small meshes replay the chunk as a CUDA graph after one eager chunk (which
  // also sets every kernel attribute outside any capture); profiling keeps
  // the eager loop so that each launch is bracketed by its events
  const bool graphs = !C->prof.on && op.nelmt < 20000;
  const std::array<uintptr_t, 26> key = {
      (uintptr_t)op.dense, (uintptr_t)op.K, (uintptr_t)op.ge, (uintptr_t)op.nelmt, (uintptr_t)op.T->d_ptr,
      (uintptr_t)op.T->d_ent, (uintptr_t)op.T->d_dof, (uintptr_t)op.T->d_pos, (uintptr_t)op.T->ngroups,
      (uintptr_t)C->d_nbr, (uintptr_t)B.Y, (uintptr_t)B.kp, (uintptr_t)B.p, (uintptr_t)B.z, (uintptr_t)B.r,
      (uintptr_t)B.cs, (uintptr_t)B.G, (uintptr_t)B.part, (uintptr_t)u, (uintptr_t)f, (uintptr_t)dp,
      (uintptr_t)n1, (uintptr_t)KR, (uintptr_t)sizeof(V), (uintptr_t)chunk, (uintptr_t)fused};
  // very small meshes with the matrix-free FP32 operator: the whole chunk as
  // one persistent cooperative launch (sg_pcg_persist.cu), below the size at
  // which the grid barrier costs more than the launches it saves
  bool persist = false;
  if constexpr (std::is_same<V, float>::value && KR <= 8)
    persist = op.dense == 2 && op.nelmt < persist_max_elements() && !C->prof.on && persist_enabled();
  int nchunks = 0;
  while (true) {
    bool done_chunk = false;
    if constexpr (std::is_same<V, float>::value)
      if (persist)
        done_chunk = launch_pcg_persistent<KR>((const float*)op.K, op.ge, op.nelmt, op.T->d_pos, *op.T, n1, u, B.r,
                                               B.z, B.p, B.kp, B.Y, dp, B.cs, B.G, B.part, chunk, s);
    cudaGraphExec_t ex = (!done_chunk && graphs && nchunks > 0) ? C->chunk_graph(key, eager_chunk) : nullptr;
    if (done_chunk) {
    } else if (ex) {
      cudaGraphLaunch(ex, s);
      add_launches((fused ? 2LL : 3LL) * chunk);
    } else {
      eager_chunk();
    }
    ++nchunks;
    cudaMemcpyAsync((void*)hG, B.G, sizeof(PcgGlobal), cudaMemcpyDeviceToHost, s);
    if (!C->check(cudaStreamSynchronize(s), "pcg")) return SG_ERR_CUDA;
    it = hG->it;
    if (hG->err) {
      // a bounded wait of this solve ran out: stop before another chunk
      status = SG_ERR_TIMEOUT;
      C->err = "PCG: a bounded wait timed out";
      break;
    }
    if (hG->all_done) break;
    if (it >= maxiter + chunk) { status = SG_ERR_TIMEOUT; break; }
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > 3600.0) { status = SG_ERR_TIMEOUT; C->err = "PCG wall-clock guard"; break; }
  }
  if constexpr (std::is_same<V, float>::value && (KR == 8 || KR == 16))
    if (fused) fused_dir_restore<KR>(n1, B.p, B.r, dp, B.cs, s);
  cudaMemcpy(hcs, B.cs, sizeof(ColState) * KR, cudaMemcpyDeviceToHost);
  for (int j = 0; j < kcols; ++j) {
    iters[j] = hcs[j].iters;
    failed[j] = hcs[j].failed;
    if (laststep) laststep[j] = std::fabs(hcs[j].alpha) * hcs[j].maxp;
    if (hcs[j].active && hcs[j].failed && status == SG_OK) status = SG_ERR_NOCONV;
  }
  if (used_iters) *used_iters = it;
  C->prof.counts[2] += it;
  return status;
}

template <typename V>
static int pcg_run(sg_ctx* C, int KR, const Op& op, const PcgBufs<V>& B, int n1, V* u, const V* f, const V* dp,
                   int kcols, const int* active, int maxiter, double tol, int mode, int* iters, int* failed,
                   int* used, double* laststep = nullptr) {
  switch (KR) {
    case 1: return pcg_run_t<V, 1>(C, op, B, n1, u, f, dp, kcols, active, maxiter, tol, mode, iters, failed, used, laststep);
    case 2: return pcg_run_t<V, 2>(C, op, B, n1, u, f, dp, kcols, active, maxiter, tol, mode, iters, failed, used, laststep);
    case 4: return pcg_run_t<V, 4>(C, op, B, n1, u, f, dp, kcols, active, maxiter, tol, mode, iters, failed, used, laststep);
    case 8: return pcg_run_t<V, 8>(C, op, B, n1, u, f, dp, kcols, active, maxiter, tol, mode, iters, failed, used, laststep);
    case 16: return pcg_run_t<V, 16>(C, op, B, n1, u, f, dp, kcols, active, maxiter, tol, mode, iters, failed, used, laststep);
  }
  return SG_ERR_BADARG;
}

// Element-apply of K (sparse layout, KR columns) followed by the plain gather:
// out = K x.  Used for warm-start products and FP64 refinement residuals.
template <typename V>
static void apply_plain(sg_ctx* C, int KR, const Op& op, const V* x, V* Y, V* out) {
  int ev = C->prof_begin();
  switch (KR) {
    case 1: pcg_apply<V, 1>(op.dense, op.K, op.ge, op.nelmt, x, (const V*)nullptr, 0, Y, nullptr, nullptr, C->d_nbr, op.T->d_pos, C->d_err, C->stream); break;
    case 2: pcg_apply<V, 2>(op.dense, op.K, op.ge, op.nelmt, x, (const V*)nullptr, 0, Y, nullptr, nullptr, C->d_nbr, op.T->d_pos, C->d_err, C->stream); break;
    case 4: pcg_apply<V, 4>(op.dense, op.K, op.ge, op.nelmt, x, (const V*)nullptr, 0, Y, nullptr, nullptr, C->d_nbr, op.T->d_pos, C->d_err, C->stream); break;
    case 8: pcg_apply<V, 8>(op.dense, op.K, op.ge, op.nelmt, x, (const V*)nullptr, 0, Y, nullptr, nullptr, C->d_nbr, op.T->d_pos, C->d_err, C->stream); break;
    case 16: pcg_apply<V, 16>(op.dense, op.K, op.ge, op.nelmt, x, (const V*)nullptr, 0, Y, nullptr, nullptr, C->d_nbr, op.T->d_pos, C->d_err, C->stream); break;
  }
  C->prof_end(ev, 1);
  ev = C->prof_begin();
  launch_gather_plain<V>(*op.T, KR, Y, out, 0, nullptr, C->stream);
  C->prof_end(ev, 2);
}

// ---------------------------------------------------------------------------
extern "C" {

sg_ctx* sg_create(int device, size_t hbm_budget) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
    cudaGetLastError();
    g_create_status = SG_ERR_NODEVICE;
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) { g_create_status = SG_ERR_NODEVICE; return nullptr; }
  sg_ctx* c = new sg_ctx();
  c->device = device;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->budget = hbm_budget ? hbm_budget : fr;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    g_create_status = SG_ERR_CUDA;
    return nullptr;
  }
  cudaMallocHost((void**)&c->pin, 4096);
  upload_constants();
  // SG_APPLY_VARIANT selects another element apply for cross-checking:
  // 0 register-staged, 1 TMA node lanes, 2 tensor cores, 3 lane apply,
  // 4 matrix-free FP32 (default 5: lane apply, matrix-free FP32 on small meshes).
  if (const char* v = std::getenv("SG_APPLY_VARIANT")) set_apply_variant(std::atoi(v));
  // SG_GATHER_VARIANT=0 selects the shared-memory-staged gather everywhere.
  if (const char* v = std::getenv("SG_GATHER_VARIANT")) set_gather_variant(std::atoi(v));
  const KsTables& T = ks_tables();
  c->d_nbr = c->alloc<int>(NGLL * KS_NBR);
  c->d_entry = c->alloc<int>(KS_NNZ);
  c->d_err = c->alloc<int>(1);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaMemcpy(c->d_nbr, T.nbr, sizeof(T.nbr), cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_entry, T.entry, sizeof(T.entry), cudaMemcpyHostToDevice);
  set_entry_table(c->d_entry);
  if (cudaGetLastError() != cudaSuccess) {
    g_create_status = SG_ERR_NODEVICE;
    delete c;
    return nullptr;
  }
  g_create_status = SG_OK;
  return c;
}

int sg_create_status(void) { return g_create_status; }

static void free_topo(sg_ctx* c, GatherTopo& T) {
  c->release(T.d_ptr); c->release(T.d_ent); c->release(T.d_dof); c->release(T.d_pos);
  T.d_ptr = T.d_ent = T.d_dof = T.d_pos = nullptr;
}

static bool upload_topo(sg_ctx* c, GatherTopo& T) {
  free_topo(c, T);
  T.d_ptr = c->alloc<int>(T.ptr.size());
  T.d_ent = c->alloc<int>(T.ent.size());
  T.d_dof = c->alloc<int>(T.dof.size());
  T.d_pos = c->alloc<int>(T.pos.size());
  if (!T.d_ptr || !T.d_ent || !T.d_dof || !T.d_pos) return false;
  if (!T.pos.empty()) cudaMemcpyAsync(T.d_pos, T.pos.data(), sizeof(int) * T.pos.size(), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(T.d_ptr, T.ptr.data(), sizeof(int) * T.ptr.size(), cudaMemcpyHostToDevice, c->stream);
  if (!T.ent.empty()) cudaMemcpyAsync(T.d_ent, T.ent.data(), sizeof(int) * T.ent.size(), cudaMemcpyHostToDevice, c->stream);
  if (!T.dof.empty()) cudaMemcpyAsync(T.d_dof, T.dof.data(), sizeof(int) * T.dof.size(), cudaMemcpyHostToDevice, c->stream);
  return true;
}

void sg_destroy(sg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->live) cudaFree(kv.first);
  c->live.clear();
  c->drop_graphs();
  for (auto& e : c->ev_pool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& e : c->marks) if (e) cudaEventDestroy(e);
  if (c->pin) cudaFreeHost(c->pin);
  cudaStreamDestroy(c->stream);
  delete c;
}

const char* sg_last_error(const sg_ctx* c) { return c ? c->err.c_str() : "no context"; }
size_t sg_hbm_used(const sg_ctx* c) { return c ? c->used : 0; }

int sg_profile_enable(sg_ctx* c, int on) {
  if (!c) return SG_ERR_BADARG;
  c->prof_flush();
  c->prof = Profile();
  c->prof.on = on != 0;
  c->launch0 = launch_count();
  return SG_OK;
}

int sg_timer_mark(sg_ctx* c, int id) {
  if (!c || id < 0 || id >= 16) return SG_ERR_BADARG;
  if (!c->marks[id]) cudaEventCreate(&c->marks[id]);
  return c->check(cudaEventRecord(c->marks[id], c->stream), "timer mark") ? SG_OK : SG_ERR_CUDA;
}

double sg_timer_ms(sg_ctx* c, int a, int b) {
  if (!c || a < 0 || b < 0 || a >= 16 || b >= 16 || !c->marks[a] || !c->marks[b]) return -1.0;
  cudaEventSynchronize(c->marks[b]);
  float ms = -1.f;
  if (cudaEventElapsedTime(&ms, c->marks[a], c->marks[b]) != cudaSuccess) return -1.0;
  return ms;
}

int sg_profile_read(sg_ctx* c, double* ms, long long* counts) {
  if (!c) return SG_ERR_BADARG;
  c->prof_flush();
  for (int i = 0; i < 8; ++i) ms[i] = c->prof.ms[i];
  for (int i = 0; i < 4; ++i) counts[i] = c->prof.counts[i];
  counts[1] = launch_count() - c->launch0;
  return SG_OK;
}

// ---------------------------------------------------------------------------
// The drop-in: pcg_solver (src/solver.f90:14-79)
// ---------------------------------------------------------------------------
int sg_pcg_solve(sg_ctx* c, int neq, int nelmt, int nedof, const double* k, double* u, const double* f,
                 const double* dprecon, const int* gdof_elmt, int cg_maxiter, double cg_tol, int* cg_iter,
                 char* errtag) {
  set_tag(errtag, "ERROR: unknown!");
  if (!c) return SG_ERR_BADARG;
  if (nedof != NEDOF || neq < 0 || nelmt < 0 || !k || !u || !f || !dprecon || !gdof_elmt || !cg_iter) {
    set_tag(errtag, "ERROR: bad argument to sg_pcg_solve (nedof must be 81)!");
    return SG_ERR_BADARG;
  }
  for (size_t i = 0; i < (size_t)nelmt * NEDOF; ++i)
    if (gdof_elmt[i] < 0 || gdof_elmt[i] > neq) {
      set_tag(errtag, "ERROR: gdof_elmt entry out of [0,neq]!");
      return SG_ERR_BADARG;
    }
  cudaSetDevice(c->device);
  auto& D = c->dropin;
  const int n1 = neq + 1;
  const size_t nk = (size_t)nelmt * NEDOF * NEDOF;
  bool same_map = (D.neq == neq && D.nelmt == nelmt &&
                   std::memcmp(D.ge.data(), gdof_elmt, sizeof(int) * (size_t)nelmt * NEDOF) == 0);
  if (!same_map) {
    D.ge.assign(gdof_elmt, gdof_elmt + (size_t)nelmt * NEDOF);
    build_groups_from_gdof(gdof_elmt, nelmt, neq, D.T);
    if (!upload_topo(c, D.T)) { set_tag(errtag, "ERROR: out of device memory!"); return SG_ERR_OOM; }
    D.neq = neq;
    D.nelmt = nelmt;
  }
  if (D.kcap < nk || D.necap < nelmt) {
    c->release(D.d_K); c->release(D.d_ge); c->release(D.Y);
    D.d_K = c->alloc<double>(nk);
    D.d_ge = c->alloc<int>((size_t)nelmt * NEDOF);
    D.Y = c->alloc<double>((size_t)nelmt * NEDOF);
    D.kcap = nk;
    D.necap = nelmt;
  }
  if (D.n1cap < n1) {
    for (double* p : {D.u, D.f, D.dp, D.r, D.z, D.p, D.kp}) c->release(p);
    D.u = c->alloc<double>(n1); D.f = c->alloc<double>(n1); D.dp = c->alloc<double>(n1);
    D.r = c->alloc<double>(n1); D.z = c->alloc<double>(n1); D.p = c->alloc<double>(n1); D.kp = c->alloc<double>(n1);
    D.n1cap = n1;
  }
  if (!D.part) {
    D.part = c->alloc<double>((size_t)NPART * 16 * 4);
    D.cs = c->alloc<ColState>(16);
    D.G = c->alloc<PcgGlobal>(1);
  }
  if (!D.d_K || !D.d_ge || !D.Y || !D.u || !D.part || !D.cs || !D.G) {
    set_tag(errtag, "ERROR: out of device memory!");
    return SG_ERR_OOM;
  }
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(D.d_K, k, sizeof(double) * nk, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.d_ge, gdof_elmt, sizeof(int) * (size_t)nelmt * NEDOF, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.u, u, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.f, f, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.dp, dprecon, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  Op op;
  op.dense = 1; op.K = D.d_K; op.ge = D.d_ge; op.nelmt = nelmt; op.T = &D.T;
  PcgBufs<double> B;
  B.r = D.r; B.z = D.z; B.p = D.p; B.kp = D.kp; B.Y = D.Y; B.part = D.part; B.cs = D.cs; B.G = D.G;
  int active = 1, it = 0, failed = 0;
  int st = pcg_run_t<double, 1>(c, op, B, n1, D.u, D.f, D.dp, 1, &active, cg_maxiter, cg_tol, 0, &it, &failed,
                                nullptr);
  cudaMemcpyAsync(u, D.u, sizeof(double) * n1, cudaMemcpyDeviceToHost, s);
  if (!c->check(cudaStreamSynchronize(s), "sg_pcg_solve")) {
    set_tag(errtag, "ERROR: CUDA failure: " + c->err);
    return SG_ERR_CUDA;
  }
  *cg_iter = it;
  if (st == SG_ERR_NOCONV) {
    set_tag(errtag, "ERROR: PCG solver doesn't converge!");
    return SG_ERR_NOCONV;
  }
  if (st != SG_OK) {
    set_tag(errtag, "ERROR: " + c->err);
    return st;
  }
  set_tag(errtag, "");
  return SG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// device-resident model
// ---------------------------------------------------------------------------
struct TrialWork {
  int KR = 0, n1 = 0, nel = 0;
  double *x = nullptr, *oldx = nullptr, *load = nullptr, *bodyload = nullptr, *Yb = nullptr;
  double *evpt = nullptr, *stress = nullptr;  // KR * nelmt_all * 27 * 6
  MatF* mf = nullptr;                          // KR * nmatblk
  PcgBufs<double> b64;
  PcgBufs<float> b32;
  // mixed form
  double *kp64 = nullptr, *r64 = nullptr;
  float *r32 = nullptr, *d32 = nullptr;
  int* colmask = nullptr;
  double* red = nullptr;
};

struct Slot {
  int used = 0;   // holds a trial (running or finished, not yet released)
  int live = 0;   // still iterating
  double dt = 0;  // pseudo-time step of the trial (dt_viscoplas)
  sg_trial_result res{};
  std::chrono::steady_clock::time_point t0;
};

struct Batch {
  bool open = false;
  sg_control ctl{};
  int kmax = 0, KR = 0;
  Slot slot[16];
  double* d_nuf = nullptr;
  bool restiff = false;
};

struct sg_model {
  sg_ctx* ctx = nullptr;
  Batch B;
  HostMesh H;
  int precision = SG_PREC_FP64;
  double* d_coord = nullptr;
  int *d_gnum = nullptr, *d_matid = nullptr, *d_ge = nullptr, *d_gdof = nullptr;
  double *d_ym = nullptr, *d_nu = nullptr, *d_gam = nullptr;
  double* d_geo = nullptr;
  GatherTopo T;
  double* d_K64 = nullptr;
  float* d_K32 = nullptr;
  float* d_rec32 = nullptr;  // matrix-free FP32 operator: per GLL point J^-1 and w detJ C (MF_REC floats)
  double *d_diag = nullptr, *d_dprecon = nullptr, *d_extload = nullptr;
  float* d_dprecon32 = nullptr;
  double* d_Yscratch = nullptr;  // nelmt*81 (diag / gravity element vectors)
  TrialWork W;
  std::vector<double> last_stress_ok;
  std::vector<double> ex_vmeps, ex_scf;  // nodal fields of the last excavation stage
  double* d_fpart = nullptr;
  double* d_wp = nullptr;  // pore pressure per node (water table set), else null
  long long plastic_steps = 0;  // batch plastic iterations run (all trials of a batch step count once)
  long long fos_steps = 0;      // of them, by the last sg_fos
};

static void model_release_work(sg_model* M) {
  sg_ctx* c = M->ctx;
  TrialWork& W = M->W;
  // W.b64.Y aliases W.Yb and W.b32.part/cs/G alias the b64 ones: released once
  for (void* p : {(void*)W.x, (void*)W.oldx, (void*)W.load, (void*)W.bodyload, (void*)W.Yb, (void*)W.evpt,
                  (void*)W.stress, (void*)W.mf, (void*)W.b64.r, (void*)W.b64.z, (void*)W.b64.p, (void*)W.b64.kp,
                  (void*)W.b64.part, (void*)W.b64.cs, (void*)W.b64.G, (void*)W.b32.r, (void*)W.b32.z,
                  (void*)W.b32.p, (void*)W.b32.kp, (void*)W.b32.Y, (void*)W.kp64, (void*)W.r64, (void*)W.r32,
                  (void*)W.d32, (void*)W.colmask, (void*)W.red})
    c->release(p);
  W = TrialWork();
}

// Allocate the per-batch workspace for KR columns (n1 dofs, nel operator elements).
static bool model_work(sg_model* M, int KR, int n1, int nel) {
  TrialWork& W = M->W;
  if (W.KR == KR && W.n1 == n1 && W.nel == nel) return true;
  model_release_work(M);
  sg_ctx* c = M->ctx;
  const size_t nv = (size_t)n1 * KR, ny = (size_t)nel * NEDOF * KR;
  const size_t ns = (size_t)KR * M->H.nelmt * NGLL * NST;
  W.KR = KR; W.n1 = n1; W.nel = nel;
  W.x = c->alloc<double>(nv); W.oldx = c->alloc<double>(nv); W.load = c->alloc<double>(nv);
  W.bodyload = c->alloc<double>(nv); W.Yb = c->alloc<double>(ny);
  W.evpt = c->alloc<double>(ns); W.stress = c->alloc<double>(ns);
  W.mf = c->alloc<MatF>((size_t)KR * M->H.nmatblk);
  W.b64.part = c->alloc<double>((size_t)NPART * 16 * 4);
  W.b64.cs = c->alloc<ColState>(16);
  W.b64.G = c->alloc<PcgGlobal>(1);
  W.red = c->alloc<double>(64);
  W.colmask = c->alloc<int>(16);
  bool ok = W.x && W.oldx && W.load && W.bodyload && W.Yb && W.evpt && W.stress && W.mf && W.b64.part && W.b64.cs &&
            W.b64.G && W.red && W.colmask;
  if (M->precision == SG_PREC_FP64) {
    W.b64.r = c->alloc<double>(nv); W.b64.z = c->alloc<double>(nv); W.b64.p = c->alloc<double>(nv);
    W.b64.kp = c->alloc<double>(nv); W.b64.Y = W.Yb;  // the apply and body-load gathers share Y
    ok = ok && W.b64.r && W.b64.z && W.b64.p && W.b64.kp;
  } else {
    W.b32.r = c->alloc<float>(nv); W.b32.z = c->alloc<float>(nv); W.b32.p = c->alloc<float>(nv);
    W.b32.kp = c->alloc<float>(nv); W.b32.Y = c->alloc<float>(ny);
    W.b32.part = W.b64.part; W.b32.cs = W.b64.cs; W.b32.G = W.b64.G;
    W.kp64 = c->alloc<double>(nv); W.r64 = c->alloc<double>(nv); W.r32 = c->alloc<float>(nv); W.d32 = c->alloc<float>(nv);
    W.b64.Y = W.Yb;
    ok = ok && W.b32.r && W.b32.z && W.b32.p && W.b32.kp && W.b32.Y && W.kp64 && W.r64 && W.r32 && W.d32;
  }
  if (!ok) model_release_work(M);
  return ok;
}

// Builds K, the diagonal preconditioner and the gravity load for the
// element list (all elements when elist is null) with Poisson ratios nuv.
static bool model_stiffness(sg_model* M, const int* d_elist, int nel, const double* d_nuv, const GatherTopo& T,
                            const int* d_ge_local, int n1, bool gravity, bool pseudoeq = true) {
  sg_ctx* c = M->ctx;
  cudaStream_t s = c->stream;
  double* Ydiag = M->d_Yscratch;
  double* Ygrav = M->d_Yscratch + (size_t)M->H.nelmt * NEDOF;
  int ev = c->prof_begin();
  launch_stiffness(M->d_geo, M->d_matid, d_elist, nel, M->d_ym, d_nuv, M->d_gam, M->d_K64, M->d_K32, Ydiag,
                   gravity ? Ygrav : nullptr, c->d_entry, T.d_pos, s, pseudoeq ? M->H.iseqload : 0, M->H.eqkx,
                   M->H.eqky, M->H.eqkz);
  launch_mf_record(M->d_geo, M->d_matid, d_elist, nel, M->d_ym, d_nuv, M->d_rec32, s);
  c->prof_end(ev, 5);
  cudaMemsetAsync(M->d_diag, 0, sizeof(double) * n1, s);
  launch_gather_plain<double>(T, 1, Ydiag, M->d_diag, 0, nullptr, s);
  cudaMemcpyAsync(M->d_dprecon, M->d_diag, sizeof(double) * n1, cudaMemcpyDeviceToDevice, s);
  launch_invert_diag(n1, M->d_dprecon, M->d_dprecon32, s);
  if (gravity) {
    cudaMemsetAsync(M->d_extload, 0, sizeof(double) * n1, s);
    launch_gather_plain<double>(T, 1, Ygrav, M->d_extload, 0, nullptr, s);
  }
  (void)d_ge_local;
  return c->check(cudaGetLastError(), "stiffness");
}

extern "C" {

static sg_model* model_build(sg_ctx* c, HostMesh&& H, int nnode8, const double* x8, const double* y8,
                             const double* z8, const int* conn8, const int* bc_counts, const int* bc_pairs,
                             int precision, char* errtag) {
  std::string err;
  cudaSetDevice(c->device);
  sg_model* M = new sg_model();
  M->ctx = c;
  M->precision = precision;
  M->H = std::move(H);
  HostMesh& h = M->H;
  if (!hex2spec(h, nnode8, x8, y8, z8, conn8, err) || !apply_bc(h, bc_counts, bc_pairs, err)) {
    set_tag(errtag, err);
    delete M;
    return nullptr;
  }
  build_gdof_elmt(h);
  build_groups_from_gdof(h.gdof_elmt.data(), h.nelmt, h.neq, M->T);
  cudaStream_t s = c->stream;
  const int ne = h.nelmt, n1 = h.neq + 1;
  M->d_coord = c->alloc<double>(h.g_coord.size());
  M->d_gnum = c->alloc<int>(h.g_num.size());
  M->d_matid = c->alloc<int>(ne);
  M->d_ge = c->alloc<int>(h.gdof_elmt.size());
  M->d_gdof = c->alloc<int>(h.gdof.size());
  M->d_ym = c->alloc<double>(h.nmatblk);
  M->d_nu = c->alloc<double>(h.nmatblk);
  M->d_gam = c->alloc<double>(h.nmatblk);
  M->d_geo = c->alloc<double>((size_t)ne * NGLL * GEO_STRIDE);
  M->d_K64 = c->alloc<double>((size_t)ne * KS_STRIDE);
  if (precision == SG_PREC_MIXED) {
    M->d_K32 = c->alloc<float>((size_t)ne * KS_STRIDE);
    M->d_rec32 = c->alloc<float>((size_t)ne * NGLL * MF_REC);
    M->d_dprecon32 = c->alloc<float>(n1);
  }
  M->d_diag = c->alloc<double>(n1);
  M->d_dprecon = c->alloc<double>(n1);
  M->d_extload = c->alloc<double>(n1);
  M->d_Yscratch = c->alloc<double>((size_t)2 * ne * NEDOF);
  M->d_fpart = c->alloc<double>(NPART * 2);
  bool ok = M->d_coord && M->d_gnum && M->d_matid && M->d_ge && M->d_gdof && M->d_ym && M->d_nu && M->d_gam &&
            M->d_geo && M->d_K64 && M->d_diag && M->d_dprecon && M->d_extload && M->d_Yscratch && M->d_fpart &&
            (precision == SG_PREC_FP64 || (M->d_K32 && M->d_rec32 && M->d_dprecon32)) && upload_topo(c, M->T);
  if (!ok) {
    set_tag(errtag, "ERROR: the model does not fit the device memory budget!");
    sg_model_free(M);
    return nullptr;
  }
  cudaMemcpyAsync(M->d_coord, h.g_coord.data(), sizeof(double) * h.g_coord.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_gnum, h.g_num.data(), sizeof(int) * h.g_num.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_matid, h.mat_id.data(), sizeof(int) * ne, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_ge, h.gdof_elmt.data(), sizeof(int) * h.gdof_elmt.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_gdof, h.gdof.data(), sizeof(int) * h.gdof.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_ym, h.ym.data(), sizeof(double) * h.nmatblk, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_nu, h.nu.data(), sizeof(double) * h.nmatblk, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->d_gam, h.gam.data(), sizeof(double) * h.nmatblk, cudaMemcpyHostToDevice, s);
  launch_geometry(M->d_coord, M->d_gnum, ne, M->d_geo, s);
  model_stiffness(M, nullptr, ne, M->d_nu, M->T, M->d_ge, n1, true);
  if (!c->check(cudaStreamSynchronize(s), "model build")) {
    set_tag(errtag, "ERROR: CUDA failure: " + c->err);
    sg_model_free(M);
    return nullptr;
  }
  set_tag(errtag, "");
  return M;
}

sg_model* sg_model_from_hex8(sg_ctx* c, int nnode8, const double* x8, const double* y8, const double* z8, int nelmt,
                             const int* conn8, const int* mat_id, int nmatblk, const double* props,
                             const int* bc_counts, const int* bc_pairs, int precision, char* errtag) {
  set_tag(errtag, "ERROR: unknown!");
  if (!c || nnode8 <= 0 || nelmt <= 0 || nmatblk <= 0 || !x8 || !y8 || !z8 || !conn8 || !mat_id || !props ||
      !bc_counts || (precision != SG_PREC_FP64 && precision != SG_PREC_MIXED)) {
    set_tag(errtag, "ERROR: bad argument to sg_model_from_hex8!");
    return nullptr;
  }
  HostMesh H;
  H.nelmt = nelmt;
  H.nmatblk = nmatblk;
  H.mat_id.assign(mat_id, mat_id + nelmt);
  for (int m : H.mat_id)
    if (m < 1 || m > nmatblk) {
      set_tag(errtag, "ERROR: material IDs must be consistent with the defined material regions!");
      return nullptr;
    }
  for (int i = 0; i < nmatblk; ++i) {
    H.gam.push_back(props[6 * i + 0]); H.ym.push_back(props[6 * i + 1]); H.nu.push_back(props[6 * i + 2]);
    H.phi.push_back(props[6 * i + 3]); H.coh.push_back(props[6 * i + 4]); H.psi.push_back(props[6 * i + 5]);
  }
  H.srf.assign(1, 1.0);
  return model_build(c, std::move(H), nnode8, x8, y8, z8, conn8, bc_counts, bc_pairs, precision, errtag);
}

static int model_set_water(sg_model* M, const std::string& wsfile, const int* water_ids, int nwmat, char* errtag);

sg_model* sg_model_from_deck(sg_ctx* c, const char* path, int precision, char* errtag) {
  set_tag(errtag, "ERROR: unknown!");
  if (!c || !path) return nullptr;
  HostMesh H;
  std::vector<double> x8, y8, z8, props;
  std::vector<int> conn, mid, cnt, pairs;
  std::string err;
  if (!read_deck(path, H, x8, y8, z8, conn, mid, props, cnt, pairs, err)) {
    set_tag(errtag, err);
    return nullptr;
  }
  H.mat_id = mid;
  for (int i = 0; i < H.nmatblk; ++i) {
    H.gam.push_back(props[6 * i + 0]); H.ym.push_back(props[6 * i + 1]); H.nu.push_back(props[6 * i + 2]);
    H.phi.push_back(props[6 * i + 3]); H.coh.push_back(props[6 * i + 4]); H.psi.push_back(props[6 * i + 5]);
  }
  const bool water = H.iswater != 0;
  const std::string wsfile = H.wsfile;
  const std::vector<int> wids = H.water_ids;
  sg_model* M = model_build(c, std::move(H), (int)x8.size(), x8.data(), y8.data(), z8.data(), conn.data(),
                            cnt.data(), pairs.data(), precision, errtag);
  if (M && water) {
    // pore pressure of the deck's water table (src/slope.F90:173-187)
    int st = model_set_water(M, wsfile, wids.data(), (int)wids.size(), errtag);
    if (st != SG_OK) { sg_model_free(M); return nullptr; }
  }
  return M;
}

// compute_pressure (src/compute_pressure.f90:10-186) on the device for the
// surfaces of a water-surface file and the given water materials; the result
// stays on the device as the model's pore pressure.
static int model_set_water(sg_model* M, const std::string& wsfile, const int* water_ids, int nwmat, char* errtag) {
  const HostMesh& h = M->H;
  std::vector<WaterSurface> surf;
  std::vector<int> face;
  std::string err;
  if (!read_wsfile(wsfile, h.nelmt, surf, face, err)) { set_tag(errtag, err); return SG_ERR_BADARG; }
  std::vector<int> wm(h.nmatblk, 0);
  for (int i = 0; i < nwmat; ++i) {
    if (water_ids[i] < 1 || water_ids[i] > h.nmatblk) {
      set_tag(errtag, "ERROR: water IDs must be consistent with the defined material regions!");
      return SG_ERR_BADARG;
    }
    wm[water_ids[i] - 1] = 1;
  }
  sg_ctx* c = M->ctx;
  cudaStream_t s = c->stream;
  if (!M->d_wp) M->d_wp = c->alloc<double>(h.nnode);
  WaterSurface* d_surf = c->alloc<WaterSurface>(surf.size() + 1);
  int* d_face = c->alloc<int>(face.size() + 2);
  int* d_wm = c->alloc<int>(wm.size() + 1);
  int* d_sub = c->alloc<int>(h.nnode);
  int* d_flag = c->alloc<int>(2);
  int st = SG_OK;
  if (!M->d_wp || !d_surf || !d_face || !d_wm || !d_sub || !d_flag) {
    set_tag(errtag, "ERROR: out of device memory!");
    st = SG_ERR_OOM;
  } else {
    cudaMemcpyAsync(d_surf, surf.data(), sizeof(WaterSurface) * surf.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_face, face.data(), sizeof(int) * face.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_wm, wm.data(), sizeof(int) * wm.size(), cudaMemcpyHostToDevice, s);
    const int flag0[2] = {INT_MAX, 0};  // smallest failing node + 1 (atomicMin), vertical-face count
    cudaMemcpyAsync(d_flag, flag0, sizeof(int) * 2, cudaMemcpyHostToDevice, s);
    launch_water_pressure(h.nnode, h.nelmt, M->d_coord, M->d_gnum, M->d_matid, d_wm, d_surf, (int)surf.size(), d_face,
                          d_sub, M->d_wp, d_flag, d_flag + 1, s);
    int flag[2] = {0, 0};
    cudaMemcpyAsync(flag, d_flag, sizeof(int) * 2, cudaMemcpyDeviceToHost, s);
    if (!c->check(cudaStreamSynchronize(s), "water pressure")) {
      set_tag(errtag, "ERROR: CUDA error in the water pressure!");
      st = SG_ERR_CUDA;
    } else if (flag[0] != INT_MAX) {
      set_tag(errtag, "ERROR: free surface cannot be determined!");
      st = SG_ERR_BADARG;
    } else if (flag[1]) {
      std::fprintf(stderr, "WARNING: free surface face is vertical! (%d nodes)\n", flag[1]);
    }
  }
  for (void* p : {(void*)d_surf, (void*)d_face, (void*)d_wm, (void*)d_sub, (void*)d_flag}) c->release(p);
  if (st != SG_OK) { c->release(M->d_wp); M->d_wp = nullptr; }
  return st;
}

int sg_model_set_water(sg_model* M, const char* wsfile, const int* water_ids, int nwmat, char* errtag) {
  set_tag(errtag, "ERROR: unknown!");
  if (!M || !wsfile || nwmat < 0 || (nwmat > 0 && !water_ids) || M->B.open) return SG_ERR_BADARG;
  int st = model_set_water(M, wsfile, water_ids, nwmat, errtag);
  if (st == SG_OK) {
    M->H.iswater = 1;
    M->H.wsfile = wsfile;
    M->H.water_ids.assign(water_ids, water_ids + nwmat);
  }
  return st;
}

int sg_model_set_pore_pressure(sg_model* M, const double* wpressure) {
  if (!M || M->B.open) return SG_ERR_BADARG;
  sg_ctx* c = M->ctx;
  if (!wpressure) {
    cudaStreamSynchronize(c->stream);
    c->release(M->d_wp);
    M->d_wp = nullptr;
    M->H.iswater = 0;
    return SG_OK;
  }
  if (!M->d_wp) M->d_wp = c->alloc<double>(M->H.nnode);
  if (!M->d_wp) return SG_ERR_OOM;
  cudaMemcpyAsync(M->d_wp, wpressure, sizeof(double) * M->H.nnode, cudaMemcpyHostToDevice, c->stream);
  M->H.iswater = 1;
  return c->check(cudaStreamSynchronize(c->stream), "pore pressure") ? SG_OK : SG_ERR_CUDA;
}

int sg_model_pore_pressure(const sg_model* M, double* wpressure) {
  if (!M || !wpressure || !M->d_wp) return SG_ERR_BADARG;
  sg_ctx* c = M->ctx;
  cudaMemcpyAsync(wpressure, M->d_wp, sizeof(double) * M->H.nnode, cudaMemcpyDeviceToHost, c->stream);
  return c->check(cudaStreamSynchronize(c->stream), "pore pressure") ? SG_OK : SG_ERR_CUDA;
}

void sg_model_free(sg_model* M) {
  if (!M) return;
  sg_ctx* c = M->ctx;
  cudaStreamSynchronize(c->stream);
  c->drop_graphs();  // captured chunks may name this model's buffers
  model_release_work(M);
  free_topo(c, M->T);
  for (void* p : {(void*)M->d_coord, (void*)M->d_gnum, (void*)M->d_matid, (void*)M->d_ge, (void*)M->d_gdof,
                  (void*)M->d_ym, (void*)M->d_nu, (void*)M->d_gam, (void*)M->d_geo, (void*)M->d_K64, (void*)M->d_K32,
                  (void*)M->d_rec32, (void*)M->d_diag, (void*)M->d_dprecon, (void*)M->d_extload, (void*)M->d_dprecon32,
                  (void*)M->d_Yscratch, (void*)M->d_fpart, (void*)M->d_wp})
    c->release(p);
  delete M;
}

int sg_model_set_eqload(sg_model* M, double eqkx, double eqky, double eqkz) {
  if (!M || M->B.open) return SG_ERR_BADARG;
  M->H.iseqload = 1;
  M->H.eqkx = eqkx; M->H.eqky = eqky; M->H.eqkz = eqkz;
  const int n1 = M->H.neq + 1;
  if (!model_stiffness(M, nullptr, M->H.nelmt, M->d_nu, M->T, M->d_ge, n1, true)) return SG_ERR_CUDA;
  return M->ctx->check(cudaStreamSynchronize(M->ctx->stream), "eqload") ? SG_OK : SG_ERR_CUDA;
}

int sg_model_info(const sg_model* M, int* info) {
  if (!M || !info) return SG_ERR_BADARG;
  info[0] = M->H.nnode; info[1] = M->H.nelmt; info[2] = M->H.neq; info[3] = M->H.nmatblk;
  info[4] = (int)M->H.srf.size(); info[5] = M->T.ngroups; info[6] = 0; info[7] = 0;
  return SG_OK;
}

int sg_model_arrays(const sg_model* M, double* g_coord, int* g_num, int* gdof, int* gdof_elmt) {
  if (!M) return SG_ERR_BADARG;
  const HostMesh& h = M->H;
  if (g_coord) std::memcpy(g_coord, h.g_coord.data(), sizeof(double) * h.g_coord.size());
  if (g_num) std::memcpy(g_num, h.g_num.data(), sizeof(int) * h.g_num.size());
  if (gdof) std::memcpy(gdof, h.gdof.data(), sizeof(int) * h.gdof.size());
  if (gdof_elmt) std::memcpy(gdof_elmt, h.gdof_elmt.data(), sizeof(int) * h.gdof_elmt.size());
  return SG_OK;
}

int sg_model_control(const sg_model* M, double* dctl, int* ictl, double* srf) {
  if (!M) return SG_ERR_BADARG;
  const HostMesh& h = M->H;
  if (dctl) { dctl[0] = h.cg_tol; dctl[1] = h.nl_tol; }
  if (ictl) { ictl[0] = h.cg_maxiter; ictl[1] = h.nl_maxiter; ictl[2] = h.phinu; ictl[3] = h.allelastic; ictl[4] = h.nexcav; ictl[5] = h.ninc; }
  if (srf) std::memcpy(srf, h.srf.data(), sizeof(double) * h.srf.size());
  return SG_OK;
}

int sg_model_stiffness(sg_model* M, double* storekm, double* dprecon, double* extload) {
  if (!M) return SG_ERR_BADARG;
  sg_ctx* c = M->ctx;
  cudaSetDevice(c->device);
  const int ne = M->H.nelmt, n1 = M->H.neq + 1;
  if (storekm) {
    double* dense = c->alloc<double>((size_t)ne * NEDOF * NEDOF);
    if (!dense) return SG_ERR_OOM;
    launch_expand_dense(M->d_K64, ne, dense, c->d_entry, c->stream);
    cudaMemcpyAsync(storekm, dense, sizeof(double) * ne * NEDOF * NEDOF, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    c->release(dense);
  }
  if (dprecon) cudaMemcpyAsync(dprecon, M->d_diag, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream);
  if (extload) cudaMemcpyAsync(extload, M->d_extload, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream);
  return c->check(cudaStreamSynchronize(c->stream), "stiffness export") ? SG_OK : SG_ERR_CUDA;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// strength reduction and pseudo-time step (host, per trial; FP64)
// ---------------------------------------------------------------------------
// strength_reduction (src/plastic_library.f90:42-88); returns istat.
static int strength_reduction(const HostMesh& h, double srf, bool phinu, std::vector<double>& cohf,
                              std::vector<double>& nuf, std::vector<double>& phif, std::vector<double>& psif) {
  const int nm = h.nmatblk;
  cohf = h.coh; nuf = h.nu; phif = h.phi; psif = h.psi;
  int istat = 0;
  if (srf != 1.0)
    for (int i = 0; i < nm; ++i) {
      phif[i] = std::atan(std::tan(h.phi[i] * DEG2RAD) / srf) * RAD2DEG;
      psif[i] = std::atan(std::tan(h.psi[i] * DEG2RAD) / srf) * RAD2DEG;
      cohf[i] = h.coh[i] / srf;
    }
  if (!phinu) return istat;
  for (int i = 0; i < nm; ++i) {
    double omtnu = 1.0 - 2.0 * h.nu[i];
    double snphif = std::sin(phif[i] * DEG2RAD);
    if (snphif < omtnu) {
      double beta = std::sin(h.phi[i] * DEG2RAD) / omtnu;
      if (beta < 1.0) beta = 1.0 + ZEROTOL;
      nuf[i] = 0.5 * (1.0 - snphif / beta);
      istat = 1;
    }
  }
  return istat;
}

// dt_viscoplas (src/plastic_library.f90:17-39)
static double dt_viscoplas(const std::vector<double>& nuf, const std::vector<double>& phif,
                           const std::vector<double>& ym, const std::vector<char>* ismat) {
  double dtm = INFTOL;
  for (size_t i = 0; i < nuf.size(); ++i) {
    if (ismat && !(*ismat)[i]) continue;
    double sn = std::sin(phif[i] * DEG2RAD);
    double dt = 4.0 * (1.0 + nuf[i]) * (1.0 - 2.0 * nuf[i]) / (ym[i] * (1.0 - 2.0 * nuf[i] + sn * sn));
    if (dt < dtm) dtm = dt;
  }
  return dtm;
}

static void make_matf(int nmat, const double* ymv, const double* nuf, const double* phif, const double* cohf,
                      const double* psif, std::vector<MatF>& out) {
  out.resize(nmat);
  for (int i = 0; i < nmat; ++i) {
    double E = ymv[i], v = nuf[i];
    double Ef = E / ((1.0 + v) * (1.0 - 2.0 * v));
    MatF& m = out[i];
    m.c11 = (1.0 - v) * Ef; m.c12 = v * Ef; m.c44 = 0.5 * (1.0 - 2.0 * v) * Ef;
    m.snph = std::sin(phif[i] * DEG2RAD); m.csph = std::cos(phif[i] * DEG2RAD);
    m.cohf = cohf[i];
    m.snps = std::sin(psif[i] * DEG2RAD);
    m.pad = 0;
  }
}

// Reads KR*nq reduced values (fixed-order device reduction) to the host.
static void reduce_read(sg_ctx* c, const double* part, int nblk, int KR, int nq, int maxmask, double* d_out,
                        double* h_out) {
  launch_final_reduce(part, nblk, KR, nq, maxmask, d_out, c->stream);
  cudaMemcpyAsync(c->pin + 256, d_out, sizeof(double) * KR * nq, cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  std::memcpy(h_out, c->pin + 256, sizeof(double) * KR * nq);
}

// ---------------------------------------------------------------------------
// Linear solve of one plastic iteration for the active columns.
// FP64: the reference PCG on the FP64 element matrices.
// MIXED: FP64 iterative refinement -- r = f - K64 x in FP64, an FP32 PCG on
// the FP32 element matrices solves K d = r to a relative residual
// inner_rtol, x += d; a column is solved when |f - K x|/|f| <= refine_rtol and
// its last correction passes the reference step test max|d|/max|x| <= cg_tol.
// ---------------------------------------------------------------------------
struct SolveStats {
  int iters[16];
  int refine = 0;
};

// The FP32 operator of the mixed solve: the stored FP32 element matrices, or
// the matrix-free form from the per-point records.
static Op fp32_op(const sg_model* M, const Op& op64) {
  Op o = op64;
  o.K = M->d_K32;
  if (fp32_matrix_free(op64.nelmt)) {
    o.dense = 2;
    o.K = M->d_rec32;
  }
  return o;
}

static int linear_solve(sg_model* M, const sg_control* ctl, const Op& op64, const Op& op32, int k,
                        const std::vector<int>& active, SolveStats& S, const double* dprecon, const float* dprecon32) {
  sg_ctx* c = M->ctx;
  TrialWork& W = M->W;
  const int KR = W.KR, n1 = W.n1;
  for (int j = 0; j < 16; ++j) S.iters[j] = 0;
  if (M->precision == SG_PREC_FP64) {
    int it[16], fl[16], used = 0;
    int st = pcg_run<double>(c, KR, op64, W.b64, n1, W.x, W.load, dprecon, k, active.data(), ctl->cg_maxiter,
                             ctl->cg_tol, 0, it, fl, &used);
    for (int j = 0; j < k; ++j) S.iters[j] = active[j] ? it[j] : 0;
    return st;
  }
  const double rtol = ctl->refine_rtol > 0 ? ctl->refine_rtol : 1e-10;
  const double itol = ctl->inner_rtol > 0 ? ctl->inner_rtol : 1e-3;
  std::vector<int> live(active);
  std::vector<int> step_ok(k, 0);
  double red[64];
  // Reliable-update mixed CG: the FP32 PCG on K32 keeps its search direction
  // across rounds; each round ends when its recursive residual has dropped by
  // itol, the correction is added to the FP64 solution, and the FP32 residual
  // is replaced by the true residual f - K64 x computed in FP64.
  for (int round = 0; round < 200; ++round) {
    apply_plain<double>(c, KR, op64, W.x, W.Yb, W.kp64);
    launch_residual_norms(n1, KR, W.load, W.kp64, W.r64, W.r32, W.b64.part, c->stream);
    reduce_read(c, W.b64.part, NPART, KR, 2, 0, W.red, red);
    S.refine++;
    c->prof.counts[3]++;
    bool any = false;
    for (int j = 0; j < k; ++j) {
      if (!live[j]) continue;
      double rr = red[2 * j], ff = red[2 * j + 1];
      bool small = ff > 0 ? std::sqrt(rr / ff) <= rtol : rr == 0.0;
      if (small && (step_ok[j] || round == 0)) live[j] = 0;
      else any = true;
    }
    if (!any) return SG_OK;
    // round 0 starts the FP32 PCG; later rounds continue its search direction
    // (all live columns enter a solve together, so they share the round structure)
    cudaMemsetAsync(W.d32, 0, sizeof(float) * (size_t)n1 * KR, c->stream);
    int it[16] = {0}, fl[16] = {0}, used = 0;
    (void)fl;
    double step[16] = {0};
    int mask[16] = {0};
    int st = pcg_run<float>(c, KR, op32, W.b32, n1, W.d32, W.r32, dprecon32, k, live.data(), ctl->cg_maxiter, itol,
                            (round == 0 ? 1 : 3) | 4, it, fl, &used, step);
    if (st != SG_OK && st != SG_ERR_NOCONV) return st;
    for (int j = 0; j < k; ++j) {
      mask[j] = live[j];
      if (live[j]) S.iters[j] += it[j];
    }
    cudaMemcpyAsync(W.colmask, mask, sizeof(int) * 16, cudaMemcpyHostToDevice, c->stream);
    launch_axpy_correction(n1, KR, W.colmask, W.d32, W.x, W.b64.part, c->stream);
    reduce_read(c, W.b64.part, NPART, KR, 2, 3, W.red, red);
    // the reference's step test on the last CG step: |alpha|*max|p| <= cg_tol*max|x|
    for (int j = 0; j < k; ++j)
      if (live[j]) step_ok[j] = (red[2 * j + 1] > 0) && (step[j] <= ctl->cg_tol * red[2 * j + 1]);
  }
  c->err = "iterative refinement did not converge";
  return SG_ERR_NOCONV;
}

// ---------------------------------------------------------------------------
// Trial batch engine: up to 16 slots, each an independent SRF trial of
// slope3d (src/slope.F90:244-443) on the model's mesh.  All live slots share
// one batched linear solve per plastic iteration (the slots are the columns
// of the multi-RHS element apply); each keeps its own factored properties,
// pseudo-time step, plastic strain, stress, body load and counters.  A slot
// freed by a finished trial can take a new trial while the others run
// (continuous batching).
// ---------------------------------------------------------------------------
static int batch_end_impl(sg_model* M);

static int batch_begin_impl(sg_model* M, const sg_control* ctl, int kmax) {
  sg_ctx* c = M->ctx;
  HostMesh& h = M->H;
  if (!ctl || kmax < 1 || kmax > 16) return SG_ERR_BADARG;
  if (ctl->precision != M->precision) {
    c->err = "control precision differs from the model's precision";
    return SG_ERR_BADARG;
  }
  if (M->B.open) batch_end_impl(M);
  cudaSetDevice(c->device);
  const int n1 = h.neq + 1, KR = next_pow2(kmax), ne = h.nelmt;
  if (!model_work(M, KR, n1, ne)) { c->err = "trial workspace does not fit the HBM budget"; return SG_ERR_OOM; }
  Batch& B = M->B;
  B = Batch();
  B.open = true;
  B.ctl = *ctl;
  B.kmax = kmax;
  B.KR = KR;
  cudaStream_t s = c->stream;
  TrialWork& W = M->W;
  const size_t nv = (size_t)n1 * KR, nst = (size_t)ne * NGLL * NST;
  cudaMemsetAsync(W.x, 0, sizeof(double) * nv, s);
  cudaMemsetAsync(W.oldx, 0, sizeof(double) * nv, s);
  cudaMemsetAsync(W.bodyload, 0, sizeof(double) * nv, s);
  cudaMemsetAsync(W.evpt, 0, sizeof(double) * nst * KR, s);
  cudaMemsetAsync(W.stress, 0, sizeof(double) * nst * KR, s);
  return c->check(cudaGetLastError(), "batch begin") ? SG_OK : SG_ERR_CUDA;
}

static int batch_add_impl(sg_model* M, double srf, int* slot_out) {
  sg_ctx* c = M->ctx;
  HostMesh& h = M->H;
  Batch& B = M->B;
  if (!B.open || srf <= 0.0) return SG_ERR_BADARG;
  int j = -1;
  for (int t = 0; t < B.kmax; ++t)
    if (!B.slot[t].used) { j = t; break; }
  if (j < 0) { c->err = "no free trial slot"; return SG_ERR_BADARG; }
  std::vector<double> cohf, nuf, phif, psif;
  int istat = strength_reduction(h, srf, B.ctl.phinu != 0, cohf, nuf, phif, psif);
  cudaStream_t s = c->stream;
  TrialWork& W = M->W;
  if (istat == 1) {
    // stiffness_bodyload is redone with the corrected Poisson ratios
    // (src/slope.F90:259-270); the batch then holds this one trial only.
    bool other = false;
    for (int t = 0; t < B.kmax; ++t) other = other || B.slot[t].used;
    if (other || B.kmax > 1) {
      c->err = "phi-nu correction changes the stiffness: run such trials one at a time";
      return SG_ERR_BADARG;
    }
    if (!B.d_nuf) B.d_nuf = c->alloc<double>(h.nmatblk);
    cudaMemcpyAsync(B.d_nuf, nuf.data(), sizeof(double) * h.nmatblk, cudaMemcpyHostToDevice, s);
    model_stiffness(M, nullptr, h.nelmt, B.d_nuf, M->T, M->d_ge, h.neq + 1, false);
    B.restiff = true;
  }
  std::vector<MatF> mf;
  make_matf(h.nmatblk, h.ym.data(), nuf.data(), phif.data(), cohf.data(), psif.data(), mf);
  cudaMemcpyAsync(W.mf + (size_t)j * h.nmatblk, mf.data(), sizeof(MatF) * h.nmatblk, cudaMemcpyHostToDevice, s);
  const int n1 = h.neq + 1;
  const size_t nst = (size_t)h.nelmt * NGLL * NST;
  launch_col_zero(n1, B.KR, j, W.x, W.oldx, W.bodyload, s);
  cudaMemsetAsync(W.evpt + nst * j, 0, sizeof(double) * nst, s);
  cudaMemsetAsync(W.stress + nst * j, 0, sizeof(double) * nst, s);
  Slot& S = B.slot[j];
  S = Slot();
  S.used = 1;
  S.live = 1;
  S.dt = dt_viscoplas(nuf, phif, h.ym, nullptr);
  S.res.srf = srf;
  S.t0 = std::chrono::steady_clock::now();
  if (slot_out) *slot_out = j;
  return c->check(cudaGetLastError(), "batch add") ? SG_OK : SG_ERR_CUDA;
}

// Nodal displacement maxima of a finished slot (src/slope.F90:400-415).
static void slot_finish(sg_model* M, int j) {
  sg_ctx* c = M->ctx;
  Slot& S = M->B.slot[j];
  double red[64];
  launch_disp_max(M->H.nnode, M->d_gdof, M->W.x, M->B.KR, j, M->W.b64.part, c->stream);
  reduce_read(c, M->W.b64.part, NPART, 1, 2, 3, M->W.red, red);
  S.res.uxmax = red[0];
  S.res.umax = red[1];
  S.res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - S.t0).count();
  S.live = 0;
}

// One plastic iteration (src/slope.F90:285-391) of every live slot.
static int batch_iteration(sg_model* M) {
  sg_ctx* c = M->ctx;
  M->plastic_steps++;
  HostMesh& h = M->H;
  Batch& B = M->B;
  TrialWork& W = M->W;
  const sg_control* ctl = &B.ctl;
  cudaStream_t s = c->stream;
  const int n1 = h.neq + 1, KR = B.KR, ne = h.nelmt, k = B.kmax;
  const size_t nst = (size_t)ne * NGLL * NST;
  std::vector<int> live(k, 0);
  bool any = false;
  for (int t = 0; t < k; ++t) { live[t] = B.slot[t].live; any = any || live[t]; }
  if (!any) return SG_OK;
  Op op64, op32;
  op64.K = M->d_K64; op64.ge = M->d_ge; op64.nelmt = ne; op64.T = &M->T;
  op32 = fp32_op(M, op64);
  launch_load_combine(n1, KR, M->d_extload, W.bodyload, W.load, s);
  SolveStats St;
  int st = linear_solve(M, ctl, op64, op32, k, live, St, M->d_dprecon, M->d_dprecon32);
  for (int t = 0; t < k; ++t) {
    if (!live[t]) continue;
    Slot& S = B.slot[t];
    S.res.nl_iter += 1;
    if (st != SG_OK) {
      // the reference stops the program on a PCG failure (error_stop, src/slope.F90:294)
      S.res.errcode = st;
      slot_finish(M, t);
      continue;
    }
    S.res.cg_tot += St.iters[t];
    S.res.refine_steps += St.refine;
  }
  if (st != SG_OK) return st;
  if (ctl->allelastic) {
    for (int t = 0; t < k; ++t) {
      if (!live[t]) continue;
      launch_elastic_stress(M->d_geo, nullptr, ne, M->d_ge, M->d_matid, W.x, KR, t, W.mf + (size_t)t * h.nmatblk, 0,
                            W.stress + nst * t, s);
      Slot& S = B.slot[t];
      S.res.failed = (S.res.nl_iter == ctl->nl_maxiter);
      slot_finish(M, t);
    }
    return SG_OK;
  }
  // uerr = max|x-oldx| / max|x|; oldx = x (src/slope.F90:307-309)
  double red[64];
  launch_nl_check(n1, KR, k, W.x, W.oldx, W.b64.part, s);
  reduce_read(c, W.b64.part, NPART, KR, 2, 3, W.red, red);
  std::vector<int> fin(k, 0), conv(k, 0);
  int gmask[16] = {0};
  bool anyg = false;
  for (int t = 0; t < k; ++t) {
    if (!live[t]) continue;
    Slot& S = B.slot[t];
    double uerr = red[2 * t] / red[2 * t + 1];
    S.res.uerr = uerr;
    conv[t] = uerr <= ctl->nl_tol;
    fin[t] = conv[t] || S.res.nl_iter == ctl->nl_maxiter;
    int ev = c->prof_begin();
    launch_stress_update(M->d_geo, nullptr, ne, M->d_ge, M->d_matid, W.x, KR, t, W.mf + (size_t)t * h.nmatblk, S.dt,
                         conv[t], fin[t], W.evpt + nst * t, W.stress + nst * t, W.Yb, KR, t, M->d_fpart, M->T.d_pos, s,
                         nullptr, nullptr, M->d_wp, M->d_gnum, 0);
    c->prof_end(ev, 4);
    reduce_read(c, M->d_fpart, NPART, 1, 1, 1, W.red, red + 32);
    S.res.fmax = red[32];
    gmask[t] = !fin[t];
    anyg = anyg || gmask[t];
  }
  // bodyload(egdof) += bload for the slots that continue
  if (anyg) {
    cudaMemcpyAsync(W.colmask, gmask, sizeof(int) * 16, cudaMemcpyHostToDevice, s);
    launch_gather_plain<double>(M->T, KR, W.Yb, W.bodyload, 1, W.colmask, s);
  }
  for (int t = 0; t < k; ++t) {
    if (!live[t] || !fin[t]) continue;
    Slot& S = B.slot[t];
    S.res.converged = conv[t];
    S.res.failed = (S.res.nl_iter == ctl->nl_maxiter);
    slot_finish(M, t);
  }
  {
    // the applies outside the PCG solves (refinement residuals) report to the
    // context's error word; it is cleared once read
    int* herr = (int*)c->pin;
    cudaMemcpyAsync(herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!c->check(cudaStreamSynchronize(s), "plastic iteration")) return SG_ERR_CUDA;
    if (*herr) {
      cudaMemsetAsync(c->d_err, 0, sizeof(int), s);
      c->err = "element apply: a bounded wait timed out";
      return SG_ERR_TIMEOUT;
    }
  }
  return c->check(cudaGetLastError(), "plastic iteration") ? SG_OK : SG_ERR_CUDA;
}

static int batch_end_impl(sg_model* M) {
  Batch& B = M->B;
  if (!B.open) return SG_OK;
  if (B.restiff) model_stiffness(M, nullptr, M->H.nelmt, M->d_nu, M->T, M->d_ge, M->H.neq + 1, false);
  M->ctx->release(B.d_nuf);
  B = Batch();
  return SG_OK;
}

static int run_trials(sg_model* M, const sg_control* ctl, int k, const double* srf, sg_trial_result* res,
                      double* x_out) {
  if (k < 1 || k > 16 || !ctl || !srf || !res) return SG_ERR_BADARG;
  int st = batch_begin_impl(M, ctl, k);
  if (st != SG_OK) return st;
  for (int t = 0; t < k && st == SG_OK; ++t) st = batch_add_impl(M, srf[t], nullptr);
  while (st == SG_OK) {
    bool any = false;
    for (int t = 0; t < k; ++t) any = any || M->B.slot[t].live;
    if (!any) break;
    st = batch_iteration(M);
  }
  for (int t = 0; t < k; ++t) res[t] = M->B.slot[t].res;
  if (x_out) {
    const int n1 = M->H.neq + 1, KR = M->B.KR;
    std::vector<double> hx((size_t)n1 * KR);
    cudaMemcpyAsync(hx.data(), M->W.x, sizeof(double) * hx.size(), cudaMemcpyDeviceToHost, M->ctx->stream);
    cudaStreamSynchronize(M->ctx->stream);
    for (int t = 0; t < k; ++t)
      for (int i = 0; i < n1; ++i) x_out[(size_t)t * n1 + i] = hx[(size_t)i * KR + t];
  }
  batch_end_impl(M);
  if (!M->ctx->check(cudaStreamSynchronize(M->ctx->stream), "trials") && st == SG_OK) st = SG_ERR_CUDA;
  return st;
}

extern "C" {

int sg_srf_trials(sg_model* M, const sg_control* ctl, int k, const double* srf, sg_trial_result* results,
                  double* x_out) {
  if (!M) return SG_ERR_BADARG;
  return run_trials(M, ctl, k, srf, results, x_out);
}

int sg_batch_begin(sg_model* M, const sg_control* ctl, int kmax) {
  return M ? batch_begin_impl(M, ctl, kmax) : SG_ERR_BADARG;
}
int sg_batch_add(sg_model* M, double srf, int* slot) { return M ? batch_add_impl(M, srf, slot) : SG_ERR_BADARG; }
int sg_batch_step(sg_model* M, int nsteps, int* nlive) {
  if (!M || !M->B.open || nsteps < 0) return SG_ERR_BADARG;
  int st = SG_OK;
  for (int i = 0; i < nsteps && st == SG_OK; ++i) {
    bool any = false;
    for (int t = 0; t < M->B.kmax; ++t) any = any || M->B.slot[t].live;
    if (!any) break;
    st = batch_iteration(M);
  }
  if (nlive) {
    int n = 0;
    for (int t = 0; t < M->B.kmax; ++t) n += M->B.slot[t].live;
    *nlive = n;
  }
  return st;
}
int sg_batch_poll(sg_model* M, int slot, sg_trial_result* res, int* state) {
  if (!M || !M->B.open || slot < 0 || slot >= M->B.kmax) return SG_ERR_BADARG;
  const Slot& S = M->B.slot[slot];
  if (res) *res = S.res;
  if (state) *state = !S.used ? 0 : (S.live ? 1 : 2);
  return SG_OK;
}
int sg_batch_release(sg_model* M, int slot) {
  if (!M || !M->B.open || slot < 0 || slot >= M->B.kmax) return SG_ERR_BADARG;
  if (M->B.slot[slot].live) return SG_ERR_BADARG;
  M->B.slot[slot] = Slot();
  return SG_OK;
}
int sg_batch_end(sg_model* M) { return M ? batch_end_impl(M) : SG_ERR_BADARG; }

int sg_last_stress(sg_model* M, int trial, double* stress_elmt) {
  if (!M || !stress_elmt || trial < 0 || trial >= M->W.KR) return SG_ERR_BADARG;
  size_t nst = (size_t)M->H.nelmt * NGLL * NST;
  cudaMemcpy(stress_elmt, M->W.stress + nst * trial, sizeof(double) * nst, cudaMemcpyDeviceToHost);
  return SG_OK;
}

int sg_excavation_fields(const sg_model* M, double* vmeps, double* scf) {
  if (!M || M->ex_vmeps.empty()) return SG_ERR_BADARG;
  if (vmeps) std::memcpy(vmeps, M->ex_vmeps.data(), sizeof(double) * M->ex_vmeps.size());
  if (scf) std::memcpy(scf, M->ex_scf.data(), sizeof(double) * M->ex_scf.size());
  return SG_OK;
}

int sg_nodal_stress(sg_model* M, int trial, double* stress_global) {
  if (!M || !stress_global || trial < 0 || trial >= M->W.KR || !M->W.stress) return SG_ERR_BADARG;
  sg_ctx* c = M->ctx;
  const HostMesh& h = M->H;
  // node -> element slots (e*27+a) in increasing element order: the order in
  // which src/slope.F90:427-431 adds the element stresses
  std::vector<int> ptr(h.nnode + 1, 0), slot((size_t)h.nelmt * NGLL);
  for (int t = 0; t < h.nelmt * NGLL; ++t) ptr[h.g_num[t] + 1]++;
  for (int n = 0; n < h.nnode; ++n) ptr[n + 1] += ptr[n];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int t = 0; t < h.nelmt * NGLL; ++t) slot[fill[h.g_num[t]]++] = t;
  int* d_ptr = c->alloc<int>(ptr.size());
  int* d_slot = c->alloc<int>(slot.size());
  double* d_out = c->alloc<double>((size_t)h.nnode * NST);
  int st = SG_OK;
  if (!d_ptr || !d_slot || !d_out) {
    st = SG_ERR_OOM;
  } else {
    cudaStream_t s = c->stream;
    cudaMemcpyAsync(d_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_slot, slot.data(), sizeof(int) * slot.size(), cudaMemcpyHostToDevice, s);
    const double* stress = M->W.stress + (size_t)trial * h.nelmt * NGLL * NST;
    launch_nodal_average(d_ptr, d_slot, h.nnode, stress, d_out, s);
    cudaMemcpyAsync(stress_global, d_out, sizeof(double) * h.nnode * NST, cudaMemcpyDeviceToHost, s);
    if (!c->check(cudaStreamSynchronize(s), "nodal stress")) st = SG_ERR_CUDA;
  }
  for (void* p : {(void*)d_ptr, (void*)d_slot, (void*)d_out}) c->release(p);
  return st;
}

int sg_srf_sweep(sg_model* M, const sg_control* ctl, int nsrf, const double* srf, sg_trial_result* results,
                 int* ndone) {
  if (!M || nsrf < 1) return SG_ERR_BADARG;
  int n = 0, st = SG_OK;
  for (int i = 0; i < nsrf; ++i) {
    st = run_trials(M, ctl, 1, srf + i, results + i, nullptr);
    ++n;
    if (st != SG_OK || results[i].failed) break;
  }
  if (ndone) *ndone = n;
  return st;
}

// Critical SRF on the grid lo + step*m, m = 0..Mg: the smallest grid SRF whose
// trial fails (the failure test of src/slope.F90:441, nl_iter == nl_maxiter),
// assuming lo is stable and hi fails, as a bisection does.
//
// k = 1: bisection, one trial at a time (sg_fos).
// k > 1 here: the k-section kept behind SG_FOS_SEARCH=ksection (sg_fos runs
// fos_speculative by default), a continuously refilled batch of k trials.  A trial that converges
// raises the stable bound a, one that fails lowers the failing bound b, and
// every running trial outside (a, b) is cancelled; each free slot takes the
// midpoint of the widest open gap between a, the running probes and b (gaps
// above the lowest running probe count half: they matter only if that probe
// converges).  Converging trials report after tens to hundreds of plastic
// iterations while failing ones take nl_maxiter, so the bracket closes from
// below while the failures are still running, and the search needs about
// two failure waits instead of one per k-section round.  Only where failure
// is monotone in SRF is the answer the bisection's.
// *ntrials = trials started, *nrounds = result events the search waited for.
static int fos_batched(sg_model* M, const sg_control* ctl, double lo, double step, int Mg, int k, int* b_out,
                       int* ntrials, int* nrounds) {
  int st = batch_begin_impl(M, ctl, k);
  if (st != SG_OK) return st;
  Batch& B = M->B;
  int a = 0, b = Mg, nt = 0, nr = 0;
  std::vector<int> idx(k, -1);   // grid index of each slot's trial, -1 free
  while (true) {
    // fill the free slots
    for (int j = 0; j < k; ++j) {
      if (idx[j] >= 0) continue;
      std::vector<int> S = {a, b};
      int low = b;
      for (int t = 0; t < k; ++t)
        if (idx[t] >= 0) { S.push_back(idx[t]); low = std::min(low, idx[t]); }
      std::sort(S.begin(), S.end());
      double best = -1.0;
      int pick = -1;
      for (size_t q = 0; q + 1 < S.size(); ++q) {
        const int g = S[q + 1] - S[q];
        if (g < 2) continue;
        const double w = g * (S[q + 1] <= low ? 1.0 : 0.5);
        if (w > best) { best = w; pick = S[q] + g / 2; }
      }
      if (pick < 0) break;
      int slot = -1;
      st = batch_add_impl(M, lo + step * pick, &slot);
      if (st != SG_OK) { batch_end_impl(M); return st; }
      idx[slot] = pick;
      ++nt;
    }
    bool any = false;
    for (int j = 0; j < k; ++j) any = any || idx[j] >= 0;
    if (!any) break;
    // plastic iterations until at least one trial has finished
    bool done = false;
    while (!done) {
      st = batch_iteration(M);
      if (st != SG_OK) { batch_end_impl(M); return st; }
      for (int j = 0; j < k; ++j) done = done || (idx[j] >= 0 && !B.slot[j].live);
    }
    ++nr;
    for (int j = 0; j < k; ++j) {
      if (idx[j] < 0 || B.slot[j].live) continue;
      const sg_trial_result& r = B.slot[j].res;
      if (r.errcode != SG_OK) { batch_end_impl(M); return r.errcode; }
      if (r.failed) b = std::min(b, idx[j]);
      else a = std::max(a, idx[j]);
      B.slot[j] = Slot();
      idx[j] = -1;
    }
    // cancel the trials that can no longer move the bracket
    for (int j = 0; j < k; ++j)
      if (idx[j] >= 0 && (idx[j] <= a || idx[j] >= b)) {
        B.slot[j] = Slot();
        idx[j] = -1;
      }
    if (b - a <= 1) break;
  }
  batch_end_impl(M);
  *b_out = b;
  if (ntrials) *ntrials = nt;
  if (nrounds) *nrounds = nr;
  return SG_OK;
}

// The bisection (k = 1 below) with its next probes run ahead in the batch.
// The probes of a bisection on [0, Mg] form a fixed tree: node (a, b) probes
// m = (a + b) / 2 and continues with (a, m) if that trial fails and with
// (m, b) if it converges.  Every free slot takes the shallowest probe of the
// current node's subtree that is neither known nor running (breadth first,
// the lower child first); a result is recorded by grid index, the current
// node descends as far as the recorded results allow, and the probes outside
// the new node's interval (the subtree not taken) are cancelled.  The
// decisions are the bisection's own, in its order, so the answer is the
// bisection's for any pattern of failures -- also where failure is not
// monotone in SRF (a trial far above the critical SRF can meet nl_tol once
// its displacement grows linearly, since uerr then falls like 1/nl_iter).
// *ntrials = trials started, *nrounds = result events waited for.
static int fos_speculative(sg_model* M, const sg_control* ctl, int Mg, double lo, double step, int k, int* b_out,
                           int* ntrials, int* nrounds) {
  int st = batch_begin_impl(M, ctl, k);
  if (st != SG_OK) return st;
  Batch& B = M->B;
  int a = 0, b = Mg, nt = 0, nr = 0;
  std::map<int, int> known;          // grid index -> 1 failed, 0 converged
  std::vector<int> idx(k, -1);       // grid index of each slot's trial, -1 free
  auto running = [&](int m) {
    for (int j = 0; j < k; ++j)
      if (idx[j] == m) return true;
    return false;
  };
  while (true) {
    while (b - a > 1) {
      auto it = known.find((a + b) / 2);
      if (it == known.end()) break;
      if (it->second) b = (a + b) / 2;
      else a = (a + b) / 2;
    }
    if (b - a <= 1) break;
    // a running probe strictly inside (a, b) belongs to this node's subtree
    for (int j = 0; j < k; ++j)
      if (idx[j] >= 0 && (idx[j] <= a || idx[j] >= b)) {
        B.slot[j] = Slot();
        idx[j] = -1;
      }
    std::vector<std::pair<int, int>> q = {{a, b}};
    for (size_t h = 0; h < q.size() && q.size() < 4096; ++h) {
      int freeslot = -1;
      for (int j = 0; j < k && freeslot < 0; ++j)
        if (idx[j] < 0 && !B.slot[j].used) freeslot = j;
      if (freeslot < 0) break;
      const int x = q[h].first, y = q[h].second;
      if (y - x <= 1) continue;
      const int m = (x + y) / 2;
      auto it = known.find(m);
      if (it == known.end() && !running(m)) {
        int slot = -1;
        st = batch_add_impl(M, lo + step * m, &slot);
        if (st != SG_OK) { batch_end_impl(M); return st; }
        idx[slot] = m;
        ++nt;
      }
      if (it == known.end() || it->second) q.push_back({x, m});
      if (it == known.end() || !it->second) q.push_back({m, y});
    }
    // plastic iterations until at least one probe has finished
    bool done = false;
    while (!done) {
      st = batch_iteration(M);
      if (st != SG_OK) { batch_end_impl(M); return st; }
      for (int j = 0; j < k; ++j) done = done || (idx[j] >= 0 && !B.slot[j].live);
    }
    ++nr;
    for (int j = 0; j < k; ++j) {
      if (idx[j] < 0 || B.slot[j].live) continue;
      const sg_trial_result& r = B.slot[j].res;
      if (r.errcode != SG_OK) { batch_end_impl(M); return r.errcode; }
      known[idx[j]] = r.failed ? 1 : 0;
      B.slot[j] = Slot();
      idx[j] = -1;
    }
  }
  batch_end_impl(M);
  *b_out = b;
  if (ntrials) *ntrials = nt;
  if (nrounds) *nrounds = nr;
  return SG_OK;
}

int sg_fos(sg_model* M, const sg_control* ctl, double lo, double hi, double step, int k, double* fos, int* ntrials,
           int* nrounds) {
  if (!M || !ctl || step <= 0 || hi <= lo || k < 1 || k > 16 || !fos) return SG_ERR_BADARG;
  const int Mg = (int)std::lround((hi - lo) / step);
  const long long steps0 = M->plastic_steps;
  if (k > 1) {
    // SG_FOS_SEARCH=ksection: the k-section search (the bisection's answer
    // only where failure is monotone in SRF); default: the batched bisection
    const char* e = std::getenv("SG_FOS_SEARCH");
    const bool ksec = e && std::strcmp(e, "ksection") == 0;
    int b = Mg;
    int st = ksec ? fos_batched(M, ctl, lo, step, Mg, k, &b, ntrials, nrounds)
                  : fos_speculative(M, ctl, Mg, lo, step, k, &b, ntrials, nrounds);
    M->fos_steps = M->plastic_steps - steps0;
    if (st != SG_OK) return st;
    *fos = lo + step * b;
    return SG_OK;
  }
  int a = 0, b = Mg, nt = 0;
  while (b - a > 1) {
    const int m = (a + b) / 2;
    const double srf = lo + step * m;
    sg_trial_result res;
    int st = run_trials(M, ctl, 1, &srf, &res, nullptr);
    ++nt;
    if (st != SG_OK) return st;
    if (res.failed) b = m;
    else a = m;
  }
  *fos = lo + step * b;
  if (ntrials) *ntrials = nt;
  if (nrounds) *nrounds = nt;
  M->fos_steps = M->plastic_steps - steps0;
  return SG_OK;
}

int sg_fos_steps(const sg_model* M, long long* steps) {
  if (!M || !steps) return SG_ERR_BADARG;
  *steps = M->fos_steps;
  return SG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// excavation3d (src/excavation.F90:15-709) with nsrf = 1
// ---------------------------------------------------------------------------
extern "C" int sg_excavation(sg_model* M, const sg_control* ctl, int s0_type, double z0, double s0, double k0,
                             int nexcav, const int* nexcavid, const int* excavid, int ninc, double srf,
                             double* stage_res, int* nstage) {
  if (!M || !ctl || nexcav < 1 || !nexcavid || !excavid || ninc < 1 || !stage_res) return SG_ERR_BADARG;
  {
    // Stage i removes excavid(id0 .. id0 + nexcavid(i) - 1) with id0 =
    // (i-1)*nexcavid(i) + 1 (src/excavation.F90:339).  With unequal counts
    // that index can pass the end of excavid (sum of nexcavid entries), where
    // the reference reads past its array; such a list is refused here.
    long long total = 0;
    for (int is = 0; is < nexcav; ++is) {
      if (nexcavid[is] < 1) { M->ctx->err = "nexcavid entries must be positive"; return SG_ERR_BADARG; }
      total += nexcavid[is];
    }
    for (int is = 0; is < nexcav; ++is)
      if ((long long)is * nexcavid[is] + nexcavid[is] > total) {
        M->ctx->err = "stage " + std::to_string(is + 1) +
                      ": (stage-1)*nexcavid(stage)+nexcavid(stage) passes the end of excavid";
        return SG_ERR_BADARG;
      }
  }
  sg_ctx* c = M->ctx;
  HostMesh& h = M->H;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int ne = h.nelmt, nm = h.nmatblk;
  const size_t nst = (size_t)ne * NGLL * NST;
  // persistent stress state
  double* stress = c->alloc<double>(nst);
  double* evpt = c->alloc<double>(nst);
  if (!stress || !evpt) { c->release(stress); c->release(evpt); return SG_ERR_OOM; }
  cudaMemsetAsync(stress, 0, sizeof(double) * nst, s);
  std::vector<double> cohf, nuf, phif, psif;
  std::vector<MatF> mf0;
  make_matf(h.nmatblk, h.ym.data(), h.nu.data(), h.phi.data(), h.coh.data(), h.psi.data(), mf0);
  MatF* d_mf = c->alloc<MatF>(nm);
  cudaMemcpyAsync(d_mf, mf0.data(), sizeof(MatF) * nm, cudaMemcpyHostToDevice, s);
  int status = SG_OK;
  if (s0_type == 1) {
    launch_overburden(M->d_coord, M->d_gnum, M->d_matid, M->d_gam, ne, z0, s0, k0, stress, s);
  } else if (s0_type == 0) {
    // gravity solve with the full mesh (src/excavation.F90:182-238)
    sg_control c0 = *ctl;
    int KR = 1, n1 = h.neq + 1;
    if (!model_work(M, KR, n1, ne)) { status = SG_ERR_OOM; goto done; }
    // the excavation's gravity load carries no pseudo-static part
    // (src/excavation.F90:191); the model's own load is restored at the end
    if (M->H.iseqload) model_stiffness(M, nullptr, ne, M->d_nu, M->T, M->d_ge, n1, true, false);
    {
      cudaMemsetAsync(M->W.x, 0, sizeof(double) * n1, s);
      cudaMemcpyAsync(M->W.load, M->d_extload, sizeof(double) * n1, cudaMemcpyDeviceToDevice, s);
      Op op64, op32;
      op64.K = M->d_K64; op64.ge = M->d_ge; op64.nelmt = ne; op64.T = &M->T;
      op32 = fp32_op(M, op64);
      SolveStats S;
      std::vector<int> act(1, 1);
      status = linear_solve(M, &c0, op64, op32, 1, act, S, M->d_dprecon, M->d_dprecon32);
      if (status != SG_OK) goto done;
      launch_elastic_stress(M->d_geo, nullptr, ne, M->d_ge, M->d_matid, M->W.x, 1, 0, d_mf, 0, stress, s);
    }
  } else {
    status = SG_ERR_BADARG;
    goto done;
  }
  {
    std::vector<char> ismat(nm, 1);
    std::vector<int> gdof = h.gdof;
    std::vector<double> nodalu((size_t)3 * h.nnode, 0.0);
    std::vector<int> ge_all((size_t)ne * NEDOF);
    int stages = 0;
    for (int is = 0; is < nexcav; ++is) {
      // id0 = (i_excav-1)*nexcavid(i_excav)+1 (src/excavation.F90:339), kept as in the reference
      int id0 = is * nexcavid[is];
      std::vector<char> off(nm, 0);
      for (int i = id0; i < id0 + nexcavid[is]; ++i) {
        if (excavid[i] < 1 || excavid[i] > nm) { status = SG_ERR_BADARG; goto done; }
        ismat[excavid[i] - 1] = 0;
        off[excavid[i] - 1] = 1;
      }
      std::vector<int> eint, evoid;
      for (int e = 0; e < ne; ++e) {
        int im = h.mat_id[e] - 1;
        if (off[im]) evoid.push_back(e);
        else if (ismat[im]) eint.push_back(e);
      }
      if (eint.empty()) break;
      std::vector<char> isnode(h.nnode, 0);
      for (int e : eint)
        for (int a = 0; a < NGLL; ++a) isnode[h.g_num[(size_t)e * NGLL + a]] = 1;
      // modify_gdof (src/excavation_library.f90:90-111)
      for (int j = 0; j < h.nnode; ++j)
        if (!isnode[j]) gdof[3 * j] = gdof[3 * j + 1] = gdof[3 * j + 2] = 0;
      int neq = 0;
      for (int j = 0; j < h.nnode; ++j)
        for (int d = 0; d < 3; ++d)
          if (gdof[3 * j + d]) gdof[3 * j + d] = ++neq;
      const int n1 = neq + 1, nint = (int)eint.size(), nvoid = (int)evoid.size();
      for (int e = 0; e < ne; ++e)
        for (int a = 0; a < NGLL; ++a)
          for (int d = 0; d < 3; ++d) ge_all[(size_t)e * NEDOF + 3 * a + d] = gdof[3 * h.g_num[(size_t)e * NGLL + a] + d];
      std::vector<int> ge_int((size_t)nint * NEDOF), ge_void((size_t)std::max(nvoid, 1) * NEDOF, 0);
      for (int i = 0; i < nint; ++i)
        std::memcpy(&ge_int[(size_t)i * NEDOF], &ge_all[(size_t)eint[i] * NEDOF], sizeof(int) * NEDOF);
      for (int i = 0; i < nvoid; ++i)
        std::memcpy(&ge_void[(size_t)i * NEDOF], &ge_all[(size_t)evoid[i] * NEDOF], sizeof(int) * NEDOF);
      GatherTopo Ti, Tv;
      build_groups_from_gdof(ge_int.data(), nint, neq, Ti);
      build_groups_from_gdof(ge_void.data(), nvoid, neq, Tv);
      int* d_eint = c->alloc<int>(nint);
      int* d_evoid = c->alloc<int>(std::max(nvoid, 1));
      int* d_geint = c->alloc<int>(ge_int.size());
      int* d_geall = c->alloc<int>(ge_all.size());
      int* d_gdofn = c->alloc<int>(gdof.size());
      // per-point effective plastic strain and safety factor of the finalize pass
      double* d_vm = c->alloc<double>((size_t)nint * NGLL);
      double* d_sf = c->alloc<double>((size_t)nint * NGLL);
      // per-stage nodal fields (src/excavation.F90:335): vmeps = 0, scf = inftol
      std::vector<double> vmeps(h.nnode, 0.0), scf(h.nnode, 1.0e32);
      bool ok = d_eint && d_evoid && d_geint && d_geall && d_gdofn && d_vm && d_sf && upload_topo(c, Ti) &&
                upload_topo(c, Tv) && model_work(M, 1, n1, nint);
      if (!ok) {
        status = SG_ERR_OOM;
      } else {
        cudaMemcpyAsync(d_eint, eint.data(), sizeof(int) * nint, cudaMemcpyHostToDevice, s);
        if (nvoid) cudaMemcpyAsync(d_evoid, evoid.data(), sizeof(int) * nvoid, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_geint, ge_int.data(), sizeof(int) * ge_int.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_geall, ge_all.data(), sizeof(int) * ge_all.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_gdofn, gdof.data(), sizeof(int) * gdof.size(), cudaMemcpyHostToDevice, s);
        TrialWork& W = M->W;
        // K9 release load of the removed elements -> extload (distribute2ghosts, src/serial_library.f90:110-130)
        double* Ye = M->d_Yscratch;
        cudaMemsetAsync(M->d_extload, 0, sizeof(double) * n1, s);
        if (nvoid) {
          launch_release_load(M->d_geo, d_evoid, nvoid, M->d_matid, M->d_gam, stress, Ye, Tv.d_pos, s);
          launch_gather_plain<double>(Tv, 1, Ye, M->d_extload, 0, nullptr, s);
        }
        launch_div((size_t)n1, M->d_extload, (double)ninc, s);
        // strength reduction, dt over the intact materials, stiffness of intact elements
        strength_reduction(h, srf, ctl->phinu != 0, cohf, nuf, phif, psif);
        double dt = dt_viscoplas(nuf, phif, h.ym, &ismat);
        std::vector<MatF> mf;
        make_matf(h.nmatblk, h.ym.data(), nuf.data(), phif.data(), cohf.data(), psif.data(), mf);
        cudaMemcpyAsync(W.mf, mf.data(), sizeof(MatF) * nm, cudaMemcpyHostToDevice, s);
        double* d_nuf = c->alloc<double>(nm);
        cudaMemcpyAsync(d_nuf, nuf.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, s);
        model_stiffness(M, d_eint, nint, d_nuf, Ti, d_geint, n1, false);
        c->release(d_nuf);
        Op op64, op32;
        op64.K = M->d_K64; op64.ge = d_geint; op64.nelmt = nint; op64.T = &Ti;
        op32 = fp32_op(M, op64);
        int cg_tot = 0, nl_tot = 0, nl_iter = 0;
        double fmax = 0.0, red[64];
        for (int inc = 0; inc < ninc && status == SG_OK; ++inc) {
          cudaMemsetAsync(W.bodyload, 0, sizeof(double) * n1, s);
          cudaMemsetAsync(evpt, 0, sizeof(double) * nst, s);
          cudaMemsetAsync(W.x, 0, sizeof(double) * n1, s);
          cudaMemsetAsync(W.oldx, 0, sizeof(double) * n1, s);
          for (nl_iter = 1; nl_iter <= ctl->nl_maxiter; ++nl_iter) {
            launch_load_combine(n1, 1, M->d_extload, W.bodyload, W.load, s);
            SolveStats S;
            std::vector<int> act(1, 1);
            int st = linear_solve(M, ctl, op64, op32, 1, act, S, M->d_dprecon, M->d_dprecon32);
            if (st != SG_OK) { status = st; break; }
            cg_tot += S.iters[0];
            launch_nl_check(n1, 1, 1, W.x, W.oldx, W.b64.part, s);
            reduce_read(c, W.b64.part, NPART, 1, 2, 3, W.red, red);
            double uerr = red[0] / red[1];
            int conv = uerr <= ctl->nl_tol, fin = conv || nl_iter == ctl->nl_maxiter;
            launch_stress_update(M->d_geo, d_eint, nint, d_geall, M->d_matid, W.x, 1, 0, W.mf, dt, conv, fin, evpt,
                                 stress, W.Yb, 1, 0, M->d_fpart, Ti.d_pos, s, d_vm, d_sf, M->d_wp, M->d_gnum, 1);
            reduce_read(c, M->d_fpart, NPART, 1, 1, 1, W.red, red);
            fmax = red[0];
            if (!fin) launch_gather_plain<double>(Ti, 1, W.Yb, W.bodyload, 1, nullptr, s);
            if (fin) {
              // vmeps(num(i)) += ..., scf(num(i)) = min(scf, sf) over the intact
              // elements in order (src/excavation.F90:597-609)
              std::vector<double> hv((size_t)nint * NGLL), hs((size_t)nint * NGLL);
              cudaMemcpy(hv.data(), d_vm, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost);
              cudaMemcpy(hs.data(), d_sf, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost);
              for (int le = 0; le < nint; ++le)
                for (int i = 0; i < NGLL; ++i) {
                  const int nd = h.g_num[(size_t)eint[le] * NGLL + i];
                  vmeps[nd] = vmeps[nd] + hv[(size_t)le * NGLL + i];
                  if (hs[(size_t)le * NGLL + i] < scf[nd]) scf[nd] = hs[(size_t)le * NGLL + i];
                }
              break;
            }
          }
          if (nl_iter > ctl->nl_maxiter) nl_iter = ctl->nl_maxiter;
          nl_tot += nl_iter;
          // nodalu += x (src/excavation.F90:631-637)
          std::vector<double> hx(n1);
          cudaMemcpy(hx.data(), W.x, sizeof(double) * n1, cudaMemcpyDeviceToHost);
          for (int j = 0; j < h.nnode; ++j)
            for (int d = 0; d < 3; ++d)
              if (gdof[3 * j + d]) nodalu[3 * j + d] += hx[gdof[3 * j + d]];
        }
        // average effective plastic strain over the intact valency (src/excavation.F90:656-661)
        {
          std::vector<int> valency(h.nnode, 0);
          for (int e : eint)
            for (int a = 0; a < NGLL; ++a) valency[h.g_num[(size_t)e * NGLL + a]]++;
          for (int j = 0; j < h.nnode; ++j)
            if (isnode[j]) vmeps[j] = vmeps[j] / (double)valency[j];
          M->ex_vmeps = vmeps;
          M->ex_scf = scf;
        }
        double uxmax = 0, umax = 0;
        for (int j = 0; j < h.nnode; ++j) {
          if (!isnode[j]) continue;
          const double* u = &nodalu[3 * j];
          for (int d = 0; d < 3; ++d) uxmax = std::max(uxmax, std::fabs(u[d]));
          umax = std::max(umax, std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
        }
        double* r = stage_res + 8 * is;
        r[0] = is + 1; r[1] = cg_tot; r[2] = nl_tot; r[3] = uxmax; r[4] = umax; r[5] = fmax;
        r[6] = (nl_iter == ctl->nl_maxiter); r[7] = status;
        ++stages;
        if (nl_iter == ctl->nl_maxiter) { /* the reference stops the stage loop */ }
      }
      free_topo(c, Ti);
      free_topo(c, Tv);
      for (void* p : {(void*)d_eint, (void*)d_evoid, (void*)d_geint, (void*)d_geall, (void*)d_gdofn, (void*)d_vm,
                      (void*)d_sf})
        c->release(p);
      if (status != SG_OK || stage_res[8 * is + 6] != 0) break;
    }
    if (nstage) *nstage = stages;
    // restore the full-mesh stiffness for later trials on this model
    model_stiffness(M, nullptr, ne, M->d_nu, M->T, M->d_ge, h.neq + 1, true);
  }
done:
  c->release(stress);
  c->release(evpt);
  c->release(d_mf);
  if (!c->check(cudaStreamSynchronize(s), "excavation") && status == SG_OK) status = SG_ERR_CUDA;
  return status;
}

// ---------------------------------------------------------------------------
// The plastic iteration's stress / yield / flow / body-load block as a host
// drop-in (src/slope.F90:311-383; excavation copy src/excavation.F90:546-616),
// for a host that keeps its own plastic loop around sg_pcg_solve.  The mesh,
// dof map, material ids and element list are uploaded (geometry computed, the
// gather topology of the listed elements built) only when they differ from the
// last call's; the plastic state goes in and out on every call.
// ---------------------------------------------------------------------------
static void release_sdrop(sg_ctx* c) {
  auto& D = c->sdrop;
  free_topo(c, D.T);
  for (void* p : {(void*)D.d_coord, (void*)D.d_geo, (void*)D.x, (void*)D.evpt, (void*)D.stress, (void*)D.bl,
                  (void*)D.Yb, (void*)D.wp, (void*)D.vm, (void*)D.sf, (void*)D.part, (void*)D.red, (void*)D.d_gnum,
                  (void*)D.d_ge, (void*)D.d_mat, (void*)D.d_elist, (void*)D.mf})
    c->release(p);
  D = sg_ctx::StressDropIn();
}

extern "C" int sg_stress_bodyload(sg_ctx* c, int neq, int nelmt, int nnode, const double* g_coord, const int* g_num,
                                  const int* gdof_elmt, const int* mat_id, int nmatblk, const double* ym_blk,
                                  const double* nuf_blk, const double* phif_blk, const double* cohf_blk,
                                  const double* psif_blk, double dt, int nl_isconv, int last, const int* elmt_list,
                                  int nel, const double* wpressure, int form, const double* x, double* evpt,
                                  double* stress_elmt, double* bodyload, double* vmeps, double* scf, double* fmax,
                                  char* errtag) {
  set_tag(errtag, "ERROR: unknown!");
  if (!c) return SG_ERR_BADARG;
  auto bad = [&](const char* m) { set_tag(errtag, m); return SG_ERR_BADARG; };
  if (neq < 0 || nelmt < 0 || nnode <= 0 || nmatblk <= 0 || (form != 0 && form != 1) || !g_coord || !g_num ||
      !gdof_elmt || !mat_id || !ym_blk || !nuf_blk || !phif_blk || !cohf_blk || !psif_blk || !x || !evpt ||
      !stress_elmt || !bodyload || !fmax)
    return bad("ERROR: bad argument to sg_stress_bodyload!");
  if (!elmt_list) nel = nelmt;
  if (nel < 0 || nel > nelmt) return bad("ERROR: element list longer than the mesh!");
  for (size_t i = 0; i < (size_t)nelmt * NGLL; ++i)
    if (g_num[i] < 1 || g_num[i] > nnode) return bad("ERROR: g_num entry out of [1,nnode]!");
  for (size_t i = 0; i < (size_t)nelmt * NEDOF; ++i)
    if (gdof_elmt[i] < 0 || gdof_elmt[i] > neq) return bad("ERROR: gdof_elmt entry out of [0,neq]!");
  for (int e = 0; e < nelmt; ++e)
    if (mat_id[e] < 1 || mat_id[e] > nmatblk) return bad("ERROR: mat_id entry out of [1,nmatblk]!");
  if (elmt_list)
    for (int i = 0; i < nel; ++i)
      if (elmt_list[i] < 1 || elmt_list[i] > nelmt) return bad("ERROR: element list entry out of [1,nelmt]!");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  auto& D = c->sdrop;
  const int n1 = neq + 1;
  const size_t nst = (size_t)NST * NGLL * nelmt;
  auto same = [](const auto& v, const auto* p, size_t n) {
    return v.size() == n && (n == 0 || std::memcmp(v.data(), p, sizeof(*p) * n) == 0);
  };
  std::vector<int> el;
  if (elmt_list) el.assign(elmt_list, elmt_list + nel);
  else { el.resize(nel); std::iota(el.begin(), el.end(), 1); }
  const bool hit = D.nnode == nnode && D.nelmt == nelmt && D.neq == neq && D.nel == nel &&
                   same(D.coord, g_coord, (size_t)3 * nnode) && same(D.gnum, g_num, (size_t)NGLL * nelmt) &&
                   same(D.ge, gdof_elmt, (size_t)NEDOF * nelmt) && same(D.mat, mat_id, (size_t)nelmt) &&
                   D.elist == el;
  if (!hit) {
    release_sdrop(c);
    D.coord.assign(g_coord, g_coord + (size_t)3 * nnode);
    D.gnum.assign(g_num, g_num + (size_t)NGLL * nelmt);
    D.ge.assign(gdof_elmt, gdof_elmt + (size_t)NEDOF * nelmt);
    D.mat.assign(mat_id, mat_id + nelmt);
    D.elist = el;
    D.d_coord = c->alloc<double>((size_t)3 * nnode);
    D.d_geo = c->alloc<double>((size_t)nelmt * NGLL * GEO_STRIDE);
    D.x = c->alloc<double>(n1); D.bl = c->alloc<double>(n1);
    D.evpt = c->alloc<double>(nst); D.stress = c->alloc<double>(nst);
    D.Yb = c->alloc<double>((size_t)nel * NEDOF);
    D.wp = c->alloc<double>(nnode);
    D.vm = c->alloc<double>((size_t)nel * NGLL); D.sf = c->alloc<double>((size_t)nel * NGLL);
    D.part = c->alloc<double>(NPART); D.red = c->alloc<double>(64);
    D.d_gnum = c->alloc<int>((size_t)NGLL * nelmt); D.d_ge = c->alloc<int>((size_t)NEDOF * nelmt);
    D.d_mat = c->alloc<int>(nelmt); D.d_elist = c->alloc<int>(nel);
    // the topology of the listed elements' dof map, element slots in list order
    std::vector<int> ge_sub((size_t)nel * NEDOF), gnum0((size_t)NGLL * nelmt), el0(nel);
    for (int i = 0; i < nel; ++i) {
      el0[i] = el[i] - 1;
      std::memcpy(&ge_sub[(size_t)i * NEDOF], gdof_elmt + (size_t)el0[i] * NEDOF, sizeof(int) * NEDOF);
    }
    for (size_t i = 0; i < gnum0.size(); ++i) gnum0[i] = g_num[i] - 1;
    build_groups_from_gdof(ge_sub.data(), nel, neq, D.T);
    bool ok = D.d_coord && D.d_geo && D.x && D.bl && D.evpt && D.stress && D.Yb && D.wp && D.vm && D.sf && D.part &&
              D.red && D.d_gnum && D.d_ge && D.d_mat && D.d_elist && upload_topo(c, D.T);
    if (!ok) {
      release_sdrop(c);
      set_tag(errtag, "ERROR: out of device memory!");
      return SG_ERR_OOM;
    }
    D.nnode = nnode; D.nelmt = nelmt; D.neq = neq; D.nel = nel;
    cudaMemcpyAsync(D.d_coord, g_coord, sizeof(double) * 3 * nnode, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(D.d_gnum, gnum0.data(), sizeof(int) * gnum0.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(D.d_ge, gdof_elmt, sizeof(int) * (size_t)NEDOF * nelmt, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(D.d_mat, mat_id, sizeof(int) * nelmt, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(D.d_elist, el0.data(), sizeof(int) * nel, cudaMemcpyHostToDevice, s);
    launch_geometry(D.d_coord, D.d_gnum, nelmt, D.d_geo, s);
    // host copies above are read by the async copies: finish them before the vectors go
    if (!c->check(cudaStreamSynchronize(s), "sg_stress_bodyload setup")) {
      release_sdrop(c);
      set_tag(errtag, "ERROR: CUDA failure: " + c->err);
      return SG_ERR_CUDA;
    }
  }
  if (D.mfcap < nmatblk) {
    c->release(D.mf);
    D.mf = c->alloc<MatF>(nmatblk);
    D.mfcap = D.mf ? nmatblk : 0;
    if (!D.mf) { set_tag(errtag, "ERROR: out of device memory!"); return SG_ERR_OOM; }
  }
  std::vector<MatF> mf;
  make_matf(nmatblk, ym_blk, nuf_blk, phif_blk, cohf_blk, psif_blk, mf);
  cudaMemcpyAsync(D.mf, mf.data(), sizeof(MatF) * nmatblk, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.x, x, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.bl, bodyload, sizeof(double) * n1, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.evpt, evpt, sizeof(double) * nst, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D.stress, stress_elmt, sizeof(double) * nst, cudaMemcpyHostToDevice, s);
  if (wpressure) cudaMemcpyAsync(D.wp, wpressure, sizeof(double) * nnode, cudaMemcpyHostToDevice, s);
  const bool fields = last && form == 1 && (vmeps || scf);
  launch_stress_update(D.d_geo, D.d_elist, nel, D.d_ge, D.d_mat, D.x, 1, 0, D.mf, dt, nl_isconv, last, D.evpt,
                       D.stress, D.Yb, 1, 0, D.part, D.T.d_pos, s, fields ? D.vm : nullptr, fields ? D.sf : nullptr,
                       wpressure ? D.wp : nullptr, D.d_gnum, form);
  double fm = 0.0;
  reduce_read(c, D.part, NPART, 1, 1, 1, D.red, &fm);
  // bodyload(egdof) += bload in element order, unless finalising; bodyload(0) = 0
  if (!last) launch_gather_plain<double>(D.T, 1, D.Yb, D.bl, 1, nullptr, s);
  cudaMemsetAsync(D.bl, 0, sizeof(double), s);
  cudaMemcpyAsync(evpt, D.evpt, sizeof(double) * nst, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(stress_elmt, D.stress, sizeof(double) * nst, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(bodyload, D.bl, sizeof(double) * n1, cudaMemcpyDeviceToHost, s);
  std::vector<double> hv, hs;
  if (fields) {
    hv.resize((size_t)nel * NGLL); hs.resize((size_t)nel * NGLL);
    cudaMemcpyAsync(hv.data(), D.vm, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hs.data(), D.sf, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, s);
  }
  if (!c->check(cudaStreamSynchronize(s), "sg_stress_bodyload")) {
    set_tag(errtag, "ERROR: CUDA failure: " + c->err);
    return SG_ERR_CUDA;
  }
  if (fields) {
    // vmeps(num(i)) += sqrt(2/3 evpt.evpt), scf(num(i)) = min(scf, sf), in
    // element-list then GLL order (src/excavation.F90:597-609)
    for (int i = 0; i < nel; ++i)
      for (int a = 0; a < NGLL; ++a) {
        const int nd = g_num[(size_t)(el[i] - 1) * NGLL + a] - 1;
        if (vmeps) vmeps[nd] = vmeps[nd] + hv[(size_t)i * NGLL + a];
        if (scf && hs[(size_t)i * NGLL + a] < scf[nd]) scf[nd] = hs[(size_t)i * NGLL + a];
      }
  }
  *fmax = fm;
  set_tag(errtag, "");
  return SG_OK;
}
