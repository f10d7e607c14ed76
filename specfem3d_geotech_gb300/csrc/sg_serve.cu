// sg_serve.cu -- device-resident request loop for factor-of-safety and
// staged-excavation solves.
//
// Requests (each its own hex8 mesh and control, with an SRF search or a list
// of excavation stages) are queued on submission and admitted in arrival
// order when their HBM footprint fits the server's budget.  Each worker thread owns a context (its own CUDA stream),
// so admitted requests run concurrently and their kernels overlap on the
// device; inside a request the SRF trials run as a continuously refilled
// batch (sg_fos: the bisection's next k probes share every element apply).
// A finished request releases its memory, which admits the next ones.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "sg_kernels.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int id = 0;
  int nnode8 = 0, nelmt = 0, nmatblk = 0;
  std::vector<double> x8, y8, z8, props;
  std::vector<int> conn8, mat_id, bc_counts, bc_pairs;
  sg_control ctl{};
  double lo = 1.0, hi = 3.0, step = 0.01;
  int k = 1;
  // kind 1: staged excavation (sg_excavation) instead of the SRF search
  int kind = 0, s0_type = 1, nexcav = 0, ninc = 1;
  double z0 = 0, s0 = 0, k0 = 0, srf = 1.0;
  std::vector<int> nexcavid, excavid;
  std::vector<double> stage_res;
  size_t footprint = 0;
  Clock::time_point t_arrival, t_start, t_done;
  int state = 0;  // 0 queued, 1 running, 2 done
  sg_fos_result res{};
};

// Device bytes of a request's model and an SRF batch of KR slots, per element
// (about 25 dofs per element on 27-node meshes): FP64 and FP32 element matrices,
// the matrix-free point records, geometry, per-slot plastic state, element
// products and vectors.
size_t estimate_footprint(int nelmt, int k, int precision) {
  const size_t kr = (size_t)(1 << (int)std::ceil(std::log2(std::max(1, k))));
  const size_t ne = (size_t)nelmt, neq = 26 * ne;
  size_t b = ne * sg::KS_STRIDE * 8 + ne * 27 * 10 * 8 + ne * 81 * 8 * 2;
  if (precision == SG_PREC_MIXED)
    b += ne * sg::KS_STRIDE * 4 + ne * sg::NGLL * sg::MF_REC * 4 + ne * 81 * kr * 4 + neq * kr * 4 * 6;
  b += kr * ne * 27 * 6 * 8 * 2 + ne * 81 * kr * 8 + neq * kr * 8 * 8 + ne * 27 * 4 * 2;
  return b + (b >> 3) + (size_t(64) << 20);
}

// An excavation request: one trial's model and plastic state plus the stage
// work arrays (the intact / void element lists and dof maps, the stage's
// gather topologies and the per-point plastic-strain and safety-factor fields).
size_t estimate_excavation_footprint(int nelmt, int precision) {
  const size_t ne = (size_t)nelmt;
  return estimate_footprint(nelmt, 1, precision) + ne * (81 * 4 * 2 + 27 * 8 * 2 + 27 * 4 * 4 + 16);
}

}  // namespace

struct sg_server {
  int device = 0;
  size_t budget = 0, used = 0;
  int next_id = 1;
  bool stop = false;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request*> queue;
  std::map<int, Request*> all;
  std::vector<std::thread> workers;
  Clock::time_point t0 = Clock::now();
  int running = 0, peak_running = 0;
};

static void worker_main(sg_server* S) {
  cudaSetDevice(S->device);
  sg_ctx* ctx = sg_create(S->device, 0);
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv.wait(lk, [&] {
        if (S->stop) return true;
        // admission in arrival order: the head of the queue runs when it fits
        return !S->queue.empty() && (S->used + S->queue.front()->footprint <= S->budget || S->running == 0);
      });
      if (S->stop && S->queue.empty()) break;
      if (S->stop) break;
      r = S->queue.front();
      S->queue.pop_front();
      S->used += r->footprint;
      r->state = 1;
      r->t_start = Clock::now();
      S->running++;
      S->peak_running = std::max(S->peak_running, S->running);
    }
    sg_fos_result res{};
    res.status = SG_ERR_NODEVICE;
    if (ctx) {
      char tag[SG_ERRTAG_LEN];
      sg_model* m = sg_model_from_hex8(ctx, r->nnode8, r->x8.data(), r->y8.data(), r->z8.data(), r->nelmt,
                                       r->conn8.data(), r->mat_id.data(), r->nmatblk, r->props.data(),
                                       r->bc_counts.data(), r->bc_pairs.data(), r->ctl.precision, tag);
      if (!m) {
        res.status = SG_ERR_BADARG;
      } else {
        int info[8];
        sg_model_info(m, info);
        res.nelmt = info[1];
        res.neq = info[2];
        if (r->kind == 1) {
          res.kind = 1;
          r->stage_res.assign((size_t)8 * r->nexcav, 0.0);
          res.status = sg_excavation(m, &r->ctl, r->s0_type, r->z0, r->s0, r->k0, r->nexcav, r->nexcavid.data(),
                                     r->excavid.data(), r->ninc, r->srf, r->stage_res.data(), &res.nstage);
          for (int st = 0; st < res.nstage; ++st) res.ntrials += (int)r->stage_res[(size_t)8 * st + 2];
        } else {
          res.status = sg_fos(m, &r->ctl, r->lo, r->hi, r->step, r->k, &res.fos, &res.ntrials, &res.nrounds);
        }
        res.hbm_bytes = (double)sg_hbm_used(ctx);
        sg_model_free(m);
      }
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      r->t_done = Clock::now();
      res.id = r->id;
      res.footprint = (double)r->footprint;
      res.t_arrival = std::chrono::duration<double>(r->t_arrival - S->t0).count();
      res.t_start = std::chrono::duration<double>(r->t_start - S->t0).count();
      res.t_done = std::chrono::duration<double>(r->t_done - S->t0).count();
      r->res = res;
      r->state = 2;
      S->used -= r->footprint;
      S->running--;
      // the mesh copy is no longer needed
      r->x8.clear(); r->y8.clear(); r->z8.clear(); r->props.clear();
      r->conn8.clear(); r->mat_id.clear(); r->bc_pairs.clear();
    }
    S->cv.notify_all();
  }
  if (ctx) sg_destroy(ctx);
}

extern "C" {

sg_server* sg_server_create(int device, size_t hbm_budget, int workers) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n || workers < 1 || workers > 64) {
    cudaGetLastError();
    return nullptr;
  }
  cudaSetDevice(device);
  sg::ks_tables();          // one-time host tables, built before any worker starts
  sg::upload_constants();
  sg_server* S = new sg_server();
  S->device = device;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  S->budget = hbm_budget ? std::min(hbm_budget, fr) : (fr / 10) * 9;
  for (int i = 0; i < workers; ++i) S->workers.emplace_back(worker_main, S);
  return S;
}

static Request* new_request(int nnode8, const double* x8, const double* y8, const double* z8, int nelmt,
                            const int* conn8, const int* mat_id, int nmatblk, const double* props,
                            const int* bc_counts, const int* bc_pairs, const sg_control* ctl) {
  Request* r = new Request();
  r->nnode8 = nnode8; r->nelmt = nelmt; r->nmatblk = nmatblk;
  r->x8.assign(x8, x8 + nnode8); r->y8.assign(y8, y8 + nnode8); r->z8.assign(z8, z8 + nnode8);
  r->conn8.assign(conn8, conn8 + (size_t)8 * nelmt);
  r->mat_id.assign(mat_id, mat_id + nelmt);
  r->props.assign(props, props + (size_t)6 * nmatblk);
  r->bc_counts.assign(bc_counts, bc_counts + 3);
  size_t npairs = (size_t)bc_counts[0] + bc_counts[1] + bc_counts[2];
  r->bc_pairs.assign(bc_pairs, bc_pairs + 2 * npairs);
  r->ctl = *ctl;
  return r;
}

static int enqueue(sg_server* S, Request* r, int* id) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (r->footprint > S->budget) { delete r; return SG_ERR_OOM; }
    r->id = S->next_id++;
    r->t_arrival = Clock::now();
    S->all[r->id] = r;
    S->queue.push_back(r);
    if (id) *id = r->id;
  }
  S->cv.notify_all();
  return SG_OK;
}

int sg_server_submit(sg_server* S, int nnode8, const double* x8, const double* y8, const double* z8, int nelmt,
                     const int* conn8, const int* mat_id, int nmatblk, const double* props, const int* bc_counts,
                     const int* bc_pairs, const sg_control* ctl, double lo, double hi, double step, int k,
                     int* id) {
  if (!S || nnode8 <= 0 || nelmt <= 0 || nmatblk <= 0 || !x8 || !y8 || !z8 || !conn8 || !mat_id || !props ||
      !bc_counts || !bc_pairs || !ctl || k < 1 || k > 16 || !(hi > lo) || !(step > 0))
    return SG_ERR_BADARG;
  Request* r = new_request(nnode8, x8, y8, z8, nelmt, conn8, mat_id, nmatblk, props, bc_counts, bc_pairs, ctl);
  r->lo = lo; r->hi = hi; r->step = step; r->k = k;
  r->footprint = estimate_footprint(nelmt, k, ctl->precision);
  return enqueue(S, r, id);
}

int sg_server_submit_excavation(sg_server* S, int nnode8, const double* x8, const double* y8, const double* z8,
                                int nelmt, const int* conn8, const int* mat_id, int nmatblk, const double* props,
                                const int* bc_counts, const int* bc_pairs, const sg_control* ctl, int s0_type,
                                double z0, double s0, double k0, int nexcav, const int* nexcavid,
                                const int* excavid, int ninc, double srf, int* id) {
  if (!S || nnode8 <= 0 || nelmt <= 0 || nmatblk <= 0 || !x8 || !y8 || !z8 || !conn8 || !mat_id || !props ||
      !bc_counts || !bc_pairs || !ctl || nexcav < 1 || !nexcavid || !excavid || ninc < 1 || !(srf > 0))
    return SG_ERR_BADARG;
  size_t nid = 0;
  for (int i = 0; i < nexcav; ++i) {
    if (nexcavid[i] < 1) return SG_ERR_BADARG;
    nid += (size_t)nexcavid[i];
  }
  Request* r = new_request(nnode8, x8, y8, z8, nelmt, conn8, mat_id, nmatblk, props, bc_counts, bc_pairs, ctl);
  r->kind = 1;
  r->s0_type = s0_type; r->z0 = z0; r->s0 = s0; r->k0 = k0;
  r->nexcav = nexcav; r->ninc = ninc; r->srf = srf;
  r->nexcavid.assign(nexcavid, nexcavid + nexcav);
  r->excavid.assign(excavid, excavid + nid);
  r->footprint = estimate_excavation_footprint(nelmt, ctl->precision);
  return enqueue(S, r, id);
}

int sg_server_stages(sg_server* S, int id, double* stage_res) {
  if (!S || !stage_res) return SG_ERR_BADARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end() || it->second->kind != 1 || it->second->state != 2) return SG_ERR_BADARG;
  const Request* r = it->second;
  std::memcpy(stage_res, r->stage_res.data(), sizeof(double) * (size_t)8 * r->res.nstage);
  return SG_OK;
}

int sg_server_wait(sg_server* S, int id, double timeout_s, sg_fos_result* out) {
  if (!S) return SG_ERR_BADARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return SG_ERR_BADARG;
  Request* r = it->second;
  bool ok = S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->state == 2; });
  if (!ok) return SG_ERR_TIMEOUT;
  if (out) *out = r->res;
  return SG_OK;
}

int sg_server_stats(sg_server* S, double* out) {
  if (!S || !out) return SG_ERR_BADARG;
  std::lock_guard<std::mutex> lk(S->mu);
  std::vector<double> lat;
  double first = 1e300, last = 0;
  for (auto& kv : S->all) {
    Request* r = kv.second;
    if (r->state != 2) continue;
    lat.push_back(r->res.t_done - r->res.t_arrival);
    first = std::min(first, r->res.t_arrival);
    last = std::max(last, r->res.t_done);
  }
  std::sort(lat.begin(), lat.end());
  auto pct = [&](double q) {
    if (lat.empty()) return 0.0;
    size_t i = (size_t)std::ceil(q * lat.size()) - 1;
    return lat[std::min(i, lat.size() - 1)];
  };
  out[0] = (double)lat.size();
  out[1] = pct(0.50);
  out[2] = pct(0.99);
  out[3] = lat.empty() ? 0.0 : lat.size() / (last - first);
  out[4] = (double)S->peak_running;
  out[5] = (double)S->budget;
  return SG_OK;
}

void sg_server_destroy(sg_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  for (auto& t : S->workers) t.join();
  for (auto& kv : S->all) delete kv.second;
  delete S;
}

}  // extern "C"
