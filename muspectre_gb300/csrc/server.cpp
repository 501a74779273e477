// Continuous-batching request server (musg_server_*), built on the library's own
// C ABI: every request becomes a cell (musg_cell_*), solved alone by musg_newton_cg
// or with requests of its kind by musg_batch_newton_cg.
//
// Admission: a lane takes the oldest waiting request whose device footprint fits the
// HBM budget next to the requests already running (a request larger than the whole
// budget is refused at submission), plus the waiting requests of the same kind
// (dimension, formulation, law kind, load steps; grids within a factor 8 in pixels)
// that fit too, up to max_batch; a batch of several grids runs grouped launches
// (requests with the consistent elasto-plastic tangent run alone, with newton_cg's
// line search).  Lanes are host threads,
// each with its own non-blocking CUDA stream, so admitted groups overlap on the
// device.  A group's memory returns to the budget when it completes.  Latency is
// measured from submission to completion on the host's steady clock.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "musg_internal.h"

using namespace musg;

namespace {

using Clock = std::chrono::steady_clock;

void need(bool ok, int code, const std::string &msg) {
  if (!ok) throw Error(code, msg);
}

int law_params(int law) { return law == MUSG_LAW_HEP1 ? 5 : (law == MUSG_LAW_LE1 || law == MUSG_LAW_LE2) ? 2 : 0; }

struct Req {
  long long id = 0;
  musg_request r{};  // pointers into the vectors below
  std::vector<int> laws;
  std::vector<double> params, per_pixel, steps;
  std::vector<unsigned char> phase;
  long long npx = 0;
  bool has_hep = false, any_le = false, has_le2 = false;
  bool has_full = false;  // an HEP1 material with the consistent tangent (D^4 tangent planes)
  unsigned long long bytes = 0;
  std::tuple<int, int, int, int, int, int, int, int, int, int, int> key;
  Clock::time_point t0;
};

unsigned long long footprint(int dim, const int *res, int form, bool has_hep, bool has_full, int precision) {
  unsigned long long npx = 1;
  for (int d = 0; d < dim; ++d) npx *= (unsigned long long)res[d];
  const unsigned long long d2 = (unsigned long long)dim * dim;
  const unsigned long long last = (unsigned long long)res[dim - 1];
  const unsigned long long nk = npx / last * (last / 2 + 1);
  // fields F, P, rhs (FP64), the FP64 spectrum, strain/stress I/O staging, material
  // index + lambda/mu, and 1 MiB of plans and reduction scratch
  unsigned long long b = 3 * d2 * npx * 8 + d2 * nk * 16 + 2 * d2 * npx * 8 + npx * (1 + 16) + (1ull << 20);
  if (form == MUSG_FINITE_STRAIN) b += 2 * d2 * npx * 8;  // S and F of the tangent
  if (has_hep) b += 38 * npx * 8;                          // plastic state
  const unsigned long long tplanes = has_full ? d2 * d2 : has_hep ? d2 * dim : 0;  // K or K'
  b += tplanes * npx * 8;
  if (precision == MUSG_PRECISION_MIXED) {
    b += npx * 8 + d2 * nk * 8 + 3 * d2 * npx * 4;  // FP32 lambda/mu, spectrum, CG vectors x r p
    b += d2 * npx * (8 + 4);                         // incremental residual: kept stress, FP32 change
    if (form == MUSG_FINITE_STRAIN) b += 2 * d2 * npx * 4;
    b += tplanes * npx * 4;
  } else {
    b += 4 * d2 * npx * 8;  // FP64 CG vectors
  }
  return b;
}

void check_request(const musg_request &r) {
  need(r.dim == 2 || r.dim == 3, MUSG_ERR_ARGUMENT, "a request needs dim 2 or 3");
  for (int d = 0; d < r.dim; ++d) need(r.resolutions[d] > 0, MUSG_ERR_ARGUMENT, "resolutions must be positive");
  need(r.formulation == MUSG_FINITE_STRAIN || r.formulation == MUSG_SMALL_STRAIN, MUSG_ERR_ARGUMENT,
       "unknown formulation");
  need(r.nb_materials >= 1 && r.nb_materials <= 256, MUSG_ERR_ARGUMENT, "a request needs 1 to 256 materials");
  need(r.laws != nullptr, MUSG_ERR_ARGUMENT, "null material laws");
  for (int m = 0; m < r.nb_materials; ++m)
    need(r.laws[m] >= MUSG_LAW_LE1 && r.laws[m] <= MUSG_LAW_HEP1, MUSG_ERR_ARGUMENT, "unknown material law");
}

bool has_law(const musg_request &r, int law) {
  for (int m = 0; m < r.nb_materials; ++m)
    if (r.laws[m] == law) return true;
  return false;
}

std::shared_ptr<Req> copy_request(const musg_request &src, int precision) {
  check_request(src);
  auto q = std::make_shared<Req>();
  const int D2 = src.dim * src.dim;
  q->npx = 1;
  for (int d = 0; d < src.dim; ++d) q->npx *= src.resolutions[d];
  need(src.phase != nullptr, MUSG_ERR_ARGUMENT, "null phase array");
  need(src.nb_steps >= 1 && src.load_steps != nullptr, MUSG_ERR_ARGUMENT, "a request needs load steps");
  q->laws.assign(src.laws, src.laws + src.nb_materials);
  q->params.assign((size_t)src.nb_materials * 5, 0.0);
  if (src.params) std::copy(src.params, src.params + (size_t)src.nb_materials * 5, q->params.begin());
  q->phase.assign(src.phase, src.phase + q->npx);
  for (unsigned char ph : q->phase)
    need(ph < src.nb_materials, MUSG_ERR_ARGUMENT, "phase index beyond the material list");
  q->has_le2 = has_law(src, MUSG_LAW_LE2);
  const bool need_pp = q->has_le2 || has_law(src, MUSG_LAW_LE3) || has_law(src, MUSG_LAW_LE4);
  if (need_pp) {
    const int want = q->has_le2 ? D2 : 2;
    need(src.per_pixel != nullptr && src.per_pixel_stride >= want, MUSG_ERR_ARGUMENT,
         "LE2/LE3/LE4 materials need per-pixel data of the right stride");
    q->per_pixel.assign(src.per_pixel, src.per_pixel + (size_t)q->npx * src.per_pixel_stride);
  }
  q->steps.assign(src.load_steps, src.load_steps + (size_t)src.nb_steps * D2);
  q->r = src;
  q->r.laws = q->laws.data();
  q->r.params = q->params.data();
  q->r.phase = q->phase.data();
  q->r.per_pixel = need_pp ? q->per_pixel.data() : nullptr;
  if (!need_pp) q->r.per_pixel_stride = 0;
  q->r.load_steps = q->steps.data();
  for (int m = 0; m < src.nb_materials; ++m) {
    if (q->laws[m] == MUSG_LAW_HEP1) {
      q->has_hep = true;
      q->has_full |= (int)q->params[5 * m + 4] == kHep1Consistent;
    } else {
      q->any_le = true;
    }
  }
  need(!(q->has_hep && src.formulation == MUSG_SMALL_STRAIN), MUSG_ERR_ARGUMENT,
       "MaterialHyperElastoPlastic1 needs the finite-strain formulation");
  int res[3] = {1, 1, 1};
  for (int d = 0; d < src.dim; ++d) res[d] = src.resolutions[d];
  q->bytes = footprint(src.dim, res, src.formulation, q->has_hep, q->has_full, precision);
  // batchable together = same dimension, formulation, flags, number of steps and
  // tangent kind (grids may differ: a batch of several grids runs grouped launches)
  q->key = std::make_tuple(src.dim, 0, 0, 0, src.formulation, src.flags, src.nb_steps, (int)q->has_hep,
                           (int)q->any_le, (int)q->has_le2, (int)q->has_full);
  return q;
}

// the cell of a request: materials in request order (empty ones skipped), on stream
musg_cell *build_cell(const Req &q, cudaStream_t stream) {
  const musg_request &r = q.r;
  const int D2 = r.dim * r.dim;
  musg_cell *cell = nullptr;
  if (musg_cell_create(r.dim, r.resolutions, r.lengths, r.formulation, r.flags, &cell) != MUSG_OK)
    throw Error(MUSG_ERR_ARGUMENT, musg_last_error());
  std::unique_ptr<musg_cell, int (*)(musg_cell *)> guard(cell, musg_cell_destroy);
  std::vector<std::vector<long long>> pix(r.nb_materials);
  for (long long p = 0; p < q.npx; ++p) pix[r.phase[p]].push_back(p);
  for (int m = 0; m < r.nb_materials; ++m) {
    if (pix[m].empty()) continue;
    const int law = r.laws[m];
    int mid = -1;
    const std::string name = "m" + std::to_string(m);
    if (musg_material_create(cell, law, name.c_str(), r.params + 5 * m, law_params(law), &mid) != MUSG_OK)
      throw Error(MUSG_ERR_ARGUMENT, musg_last_error());
    const int stride = law == MUSG_LAW_LE2 ? D2 : (law == MUSG_LAW_LE3 || law == MUSG_LAW_LE4) ? 2 : 0;
    std::vector<double> pp;
    if (stride) {
      pp.resize(pix[m].size() * (size_t)stride);
      for (size_t k = 0; k < pix[m].size(); ++k)
        std::memcpy(&pp[k * stride], r.per_pixel + (size_t)pix[m][k] * r.per_pixel_stride, stride * sizeof(double));
    }
    if (musg_material_add_pixels(cell, mid, pix[m].data(), (long long)pix[m].size(), stride ? pp.data() : nullptr,
                                 stride) != MUSG_OK)
      throw Error(MUSG_ERR_ARGUMENT, musg_last_error());
  }
  if (musg_cell_set_stream(cell, stream) != MUSG_OK) throw Error(MUSG_ERR_CUDA, musg_last_error());
  if (musg_cell_initialise(cell, 0) != MUSG_OK) throw Error(MUSG_ERR_RUNTIME, musg_last_error());
  return guard.release();
}

void set_message(musg_server_result &res, const std::string &m) {
  std::strncpy(res.message, m.c_str(), sizeof(res.message) - 1);
  res.message[sizeof(res.message) - 1] = 0;
}

}  // namespace

struct musg_server {
  unsigned long long budget = 0, in_use = 0, peak = 0;
  int lanes = 0, max_batch = 1, precision = MUSG_PRECISION_MIXED;
  double tol = 1e-8, newton_tol = 1e-6;
  unsigned maxiter = 1000;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Req>> queue;
  std::map<long long, musg_server_result> done;
  long long next_id = 1, submitted = 0, completed = 0, batches = 0;
  bool closed = false;
  std::vector<std::thread> threads;
  std::vector<std::shared_ptr<int>> running;  // stop flags of the groups being solved

  // the admission step (caller holds mu)
  std::vector<std::shared_ptr<Req>> take(unsigned long long &used) {
    std::vector<std::shared_ptr<Req>> group;
    used = 0;
    for (size_t i = 0; i < queue.size(); ++i) {
      const auto &q = queue[i];
      if (in_use + q->bytes > budget) continue;
      group.push_back(q);
      used = q->bytes;
      // requests solved with the line search (consistent elasto-plastic tangent) run alone
      for (size_t k = i + 1; k < queue.size() && (int)group.size() < max_batch && !q->has_full; ++k) {
        const auto &o = queue[k];
        // grids within a factor 8 in pixels of the first: the batch's Newton steps run
        // in lockstep, so a much larger cell would hold the smaller ones back
        const bool close = o->npx <= 8 * q->npx && q->npx <= 8 * o->npx;
        if (o->key == q->key && close && in_use + used + o->bytes <= budget) {
          group.push_back(o);
          used += o->bytes;
        }
      }
      break;
    }
    for (const auto &g : group) queue.erase(std::find(queue.begin(), queue.end(), g));
    in_use += used;
    peak = std::max(peak, in_use);
    return group;
  }

  std::vector<musg_server_result> run(const std::vector<std::shared_ptr<Req>> &group, cudaStream_t stream,
                                      const int *stop) {
    const int n = (int)group.size();
    std::vector<musg_server_result> out(n);
    for (int k = 0; k < n; ++k) {
      std::memset(&out[k], 0, sizeof(out[k]));
      out[k].id = group[k]->id;
      out[k].batched_with = n;
    }
    std::vector<musg_cell *> cells(n, nullptr);
    auto cleanup = [&]() {
      for (musg_cell *c : cells)
        if (c) musg_cell_destroy(c);
    };
    try {
      for (int k = 0; k < n; ++k) cells[k] = build_cell(*group[k], stream);
      const int ns = group[0]->r.nb_steps;
      const int D2 = group[0]->r.dim * group[0]->r.dim;
      std::vector<musg_result_info> infos((size_t)n * ns);
      std::memset(infos.data(), 0, infos.size() * sizeof(musg_result_info));
      std::vector<int> rc(n, MUSG_OK);
      std::vector<std::string> err(n);
      if (n == 1) {
        musg_solver *sv = nullptr;
        if (musg_solver_cg_create(cells[0], tol, maxiter, 0, precision, &sv) != MUSG_OK)
          throw Error(MUSG_ERR_RUNTIME, musg_last_error());
        // the consistent elasto-plastic tangent converges with the line search
        musg_solver_set_line_search(sv, group[0]->has_full ? 1 : 0);
        musg_solver_set_stop_flag(sv, stop);
        rc[0] = musg_newton_cg(cells[0], group[0]->steps.data(), ns, sv, newton_tol, 0.0, 0, infos.data(), nullptr,
                               nullptr);
        if (rc[0] != MUSG_OK) err[0] = musg_last_error();
        musg_solver_destroy(sv);
      } else {
        std::vector<double> steps((size_t)n * ns * D2);
        for (int k = 0; k < n; ++k) std::copy(group[k]->steps.begin(), group[k]->steps.end(), steps.begin() + (size_t)k * ns * D2);
        musg_batch *b = nullptr;
        if (musg_batch_create(cells.data(), n, tol, maxiter, precision, &b) != MUSG_OK)
          throw Error(MUSG_ERR_RUNTIME, musg_last_error());
        musg_batch_set_stop_flag(b, stop);
        const int brc = musg_batch_newton_cg(b, steps.data(), ns, newton_tol, 0.0, infos.data(), nullptr);
        const std::string berr = brc == MUSG_OK ? "" : musg_last_error();
        musg_batch_destroy(b);
        if (brc != MUSG_OK) throw Error(brc, berr);
      }
      for (int k = 0; k < n; ++k) {
        musg_server_result &res = out[k];
        int okc = 0;
        for (int s = 0; s < ns; ++s) okc += infos[(size_t)k * ns + s].success ? 1 : 0;
        res.nb_steps_done = okc;
        res.success = rc[k] == MUSG_OK && okc == ns;
        const musg_result_info &last = infos[(size_t)k * ns + ns - 1];
        res.nb_it = last.nb_it;
        res.nb_fev = last.nb_fev;
        if (rc[k] != MUSG_OK) set_message(res, err[k]);
        else set_message(res, last.message);
        for (int c = 0; c < 9; ++c) res.stress[c] = 0.0;
        // the homogenised stress at the returned strain: an FP64 newton_cg leaves the
        // stress of its last evaluation, one Newton increment earlier, so history-free
        // cells are evaluated once more (a mixed solve already did that)
        if (res.success && precision == MUSG_PRECISION_FP64 && !group[k]->has_hep &&
            musg_cell_evaluate_stress_tangent(cells[k], nullptr, nullptr) != MUSG_OK) {
          res.success = 0;
          set_message(res, musg_last_error());
        }
        if (res.success && musg_cell_homogenised_stress(cells[k], res.stress) != MUSG_OK) {
          res.success = 0;
          set_message(res, musg_last_error());
        }
      }
    } catch (const std::exception &e) {
      for (auto &res : out) {
        res.success = 0;
        set_message(res, e.what());
      }
    }
    cleanup();
    return out;
  }

  void lane() {
    cudaStream_t stream = nullptr;
    if (musg_set_device(device) != MUSG_OK || cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) {
      stream = nullptr;
    }
    for (;;) {
      std::vector<std::shared_ptr<Req>> group;
      unsigned long long used = 0;
      // the group's stop flag is registered in the same critical section that admits
      // it, so musg_server_cancel_running reaches every admitted group
      auto stop = std::make_shared<int>(0);
      {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
          group = take(used);
          if (!group.empty()) {
            running.push_back(stop);
            break;
          }
          if (closed && queue.empty()) {
            if (stream) cudaStreamDestroy(stream);
            return;
          }
          cv.wait(lk);
        }
      }
      std::vector<musg_server_result> res;
      const Clock::time_point ta = Clock::now();
      if (stream) {
        res = run(group, stream, stop.get());
      } else {
        res.resize(group.size());
        for (size_t k = 0; k < group.size(); ++k) {
          std::memset(&res[k], 0, sizeof(res[k]));
          res[k].id = group[k]->id;
          set_message(res[k], "the lane has no CUDA stream");
        }
      }
      const Clock::time_point t1 = Clock::now();
      {
        std::lock_guard<std::mutex> lk(mu);
        in_use -= used;
        running.erase(std::find(running.begin(), running.end(), stop));
        for (size_t k = 0; k < res.size(); ++k) {
          res[k].latency_s = std::chrono::duration<double>(t1 - group[k]->t0).count();
          res[k].service_s = std::chrono::duration<double>(t1 - ta).count();
          done[res[k].id] = res[k];
        }
        completed += (long long)res.size();
        if (group.size() > 1) batches += 1;
      }
      cv.notify_all();
    }
  }
};

extern "C" {

int musg_request_bytes(const musg_request *req, int precision, unsigned long long *bytes) {
  return guarded([&] {
    need(req && bytes, MUSG_ERR_ARGUMENT, "null argument");
    check_request(*req);
    int res[3] = {1, 1, 1};
    for (int d = 0; d < req->dim; ++d) res[d] = req->resolutions[d];
    bool full = false;
    for (int m = 0; m < req->nb_materials; ++m)
      full |= req->laws[m] == MUSG_LAW_HEP1 && req->params && (int)req->params[5 * m + 4] == kHep1Consistent;
    *bytes = footprint(req->dim, res, req->formulation, has_law(*req, MUSG_LAW_HEP1), full, precision);
  });
}

int musg_server_create(unsigned long long hbm_budget, int lanes, int max_batch, int precision, double tol,
                       unsigned maxiter, double newton_tol, musg_server **out) {
  return guarded([&] {
    need(out != nullptr, MUSG_ERR_ARGUMENT, "null output handle");
    need(lanes >= 0 && lanes <= 64, MUSG_ERR_ARGUMENT, "0 to 64 lanes");
    need(max_batch >= 1, MUSG_ERR_ARGUMENT, "max_batch must be at least 1");
    need(precision == MUSG_PRECISION_FP64 || precision == MUSG_PRECISION_MIXED, MUSG_ERR_ARGUMENT,
         "unknown precision");
    auto s = std::make_unique<musg_server>();
    s->budget = hbm_budget;
    s->lanes = lanes;
    s->max_batch = max_batch;
    s->precision = precision;
    s->tol = tol;
    s->maxiter = maxiter;
    s->newton_tol = newton_tol;
    if (lanes > 0) {
      MUSG_CUDA(cudaGetDevice(&s->device));
      for (int k = 0; k < lanes; ++k) s->threads.emplace_back([p = s.get()] { p->lane(); });
    }
    *out = s.release();
  });
}

int musg_server_submit(musg_server *srv, const musg_request *req, long long *id) {
  return guarded([&] {
    need(srv && req, MUSG_ERR_ARGUMENT, "null argument");
    auto q = copy_request(*req, srv->precision);
    // a request that cannot fit the budget even on an idle server is refused here,
    // instead of being admitted alone and overcommitting the device
    if (q->bytes > srv->budget)
      throw Error(MUSG_ERR_MEMORY, "request needs " + std::to_string(q->bytes) + " bytes of device memory, above the "
                                       "server's HBM budget of " + std::to_string(srv->budget) + " bytes");
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      need(!srv->closed, MUSG_ERR_RUNTIME, "the server is closed");
      q->id = srv->next_id++;
      q->t0 = Clock::now();
      srv->queue.push_back(q);
      srv->submitted += 1;
    }
    if (id) *id = q->id;
    srv->cv.notify_all();
  });
}

int musg_server_close(musg_server *srv) {
  return guarded([&] {
    need(srv != nullptr, MUSG_ERR_ARGUMENT, "null server");
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->closed = true;
    }
    srv->cv.notify_all();
  });
}

int musg_server_cancel_waiting(musg_server *srv, long long *cancelled) {
  return guarded([&] {
    need(srv != nullptr, MUSG_ERR_ARGUMENT, "null server");
    long long n = 0;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      const Clock::time_point t1 = Clock::now();
      for (const auto &q : srv->queue) {
        musg_server_result res;
        std::memset(&res, 0, sizeof(res));
        res.id = q->id;
        res.latency_s = std::chrono::duration<double>(t1 - q->t0).count();
        set_message(res, "cancelled before admission");
        srv->done[q->id] = res;
        ++n;
      }
      srv->queue.clear();
      srv->completed += n;
    }
    srv->cv.notify_all();
    if (cancelled) *cancelled = n;
  });
}

int musg_server_cancel_running(musg_server *srv, long long *groups) {
  return guarded([&] {
    need(srv != nullptr, MUSG_ERR_ARGUMENT, "null server");
    long long n = 0;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      for (const auto &f : srv->running) {
        __atomic_store_n(f.get(), 1, __ATOMIC_RELAXED);
        ++n;
      }
    }
    if (groups) *groups = n;
  });
}

int musg_server_wait(musg_server *srv, long long id, double timeout_s, musg_server_result *out) {
  return guarded([&] {
    need(srv && out, MUSG_ERR_ARGUMENT, "null argument");
    std::unique_lock<std::mutex> lk(srv->mu);
    need(id >= 1 && id < srv->next_id, MUSG_ERR_ARGUMENT, "unknown request id");
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(
                                          std::max(0.0, timeout_s)));
    while (!srv->done.count(id)) {
      if (srv->cv.wait_until(lk, until) == std::cv_status::timeout && !srv->done.count(id))
        throw Error(MUSG_ERR_RUNTIME, "request " + std::to_string(id) + " is not done (or was fetched already)");
    }
    *out = srv->done[id];
    srv->done.erase(id);
  });
}

int musg_server_get_stats(musg_server *srv, musg_server_stats *out) {
  return guarded([&] {
    need(srv && out, MUSG_ERR_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    out->submitted = srv->submitted;
    out->completed = srv->completed;
    out->batches = srv->batches;
    out->budget = srv->budget;
    out->in_use = srv->in_use;
    out->peak_in_use = srv->peak;
    out->queued = (long long)srv->queue.size();
  });
}

int musg_server_destroy(musg_server *srv) {
  return guarded([&] {
    if (!srv) return;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->closed = true;
    }
    srv->cv.notify_all();
    for (auto &t : srv->threads) t.join();
    delete srv;
  });
}

int musg_server_admit(musg_server *srv, long long *ids, int cap, int *count, unsigned long long *bytes) {
  return guarded([&] {
    need(srv && ids && count && bytes && cap >= 1, MUSG_ERR_ARGUMENT, "null argument");
    need(srv->lanes == 0, MUSG_ERR_ARGUMENT, "admission by hand needs a server without lanes");
    std::lock_guard<std::mutex> lk(srv->mu);
    const int keep = srv->max_batch;
    srv->max_batch = std::min(srv->max_batch, cap);
    unsigned long long used = 0;
    auto g = srv->take(used);
    srv->max_batch = keep;
    *count = (int)g.size();
    *bytes = used;
    for (size_t k = 0; k < g.size(); ++k) ids[k] = g[k]->id;
  });
}

int musg_server_release(musg_server *srv, unsigned long long bytes) {
  return guarded([&] {
    need(srv != nullptr, MUSG_ERR_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(srv->mu);
    need(bytes <= srv->in_use, MUSG_ERR_ARGUMENT, "releasing more than is in use");
    srv->in_use -= bytes;
  });
}

}  // extern "C"
