// Continuous-batching scheduler over size classes (mhd_server_* of include/mhdgb.h), built only on
// the library's public batch entry points: a size class is a batch handle (mhd_batch_create) whose
// active slots step together; every class steps on its own stream, so the classes of one tick run
// concurrently on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <map>
#include <string>
#include <vector>

#include "../../include/mhdgb.h"

namespace mhdgb {
int report_error(int code, const std::string& msg);
}

namespace {

const int kSizes[8] = {16, 32, 48, 64, 96, 128, 256, 512};
const int kDefaultCapacity[8] = {32, 32, 24, 16, 8, 8, 4, 1};

int size_index(int n) {
  for (int i = 0; i < 8; ++i)
    if (kSizes[i] == n) return i;
  return -1;
}

struct Request {
  mhd_request r{};
  std::vector<float> init;    // (nkr, n, n, 6) complex64 as float pairs
  std::vector<float> result;  // final state (keep_states)
  double diag[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int status = MHD_REQ_QUEUED;
  long long done = 0;
  std::string error;
  int code = MHD_OK;  // status code mhd_server_result returns for a failed / rejected request
  int cls = -1;  // index into classes
  int slot = -1;
};

struct SizeClass {
  mhd_handle h = nullptr;
  int n = 0;
  double L = 0;
  int cap = 0;
  double bytes = 0;
};

}  // namespace

struct mhd_server_s {
  mhd_server_params p{};
  std::map<long long, Request> reqs;
  std::deque<long long> queued;   // arrival order
  std::vector<long long> active;
  std::vector<SizeClass> classes;
  double reserved = 0, peak = 0;
  long long next = 1;

  ~mhd_server_s() {
    for (auto& c : classes)
      if (c.h) mhd_destroy(c.h);
  }

  int capacity_of(int n) const {
    const int i = size_index(n);
    return (i >= 0 && p.capacity[i] > 0) ? p.capacity[i] : (i >= 0 ? kDefaultCapacity[i] : 1);
  }
  mhd_params params_of(int n, double L) const {
    mhd_params q{};
    q.n = n;
    q.L = L;
    q.scheme = p.scheme;
    q.device = p.device;
    return q;
  }
  // device bytes of a class of n with cap slots (0 when the size is not supported)
  double class_bytes(int n, double L, int cap) const {
    const mhd_params q = params_of(n, L);
    long long per_slot = 0, per_class = 0;
    if (mhd_slot_bytes(&q, &per_slot, &per_class) != MHD_OK) return 0;
    return (double)per_class + (double)cap * (double)per_slot;
  }
  int free_class(int n, double L) const {
    for (size_t i = 0; i < classes.size(); ++i) {
      const SizeClass& c = classes[i];
      if (!c.h || c.n != n || c.L != L) continue;
      int capv = 0, act = 0;
      if (mhd_batch_info(c.h, &capv, &act) == MHD_OK && act < capv) return (int)i;
    }
    return -1;
  }
  // release size classes without active slots (their memory goes back to the budget)
  void reclaim() {
    for (auto& c : classes) {
      if (!c.h) continue;
      int capv = 0, act = 0;
      if (mhd_batch_info(c.h, &capv, &act) == MHD_OK && act == 0) {
        mhd_destroy(c.h);
        c.h = nullptr;
        reserved -= c.bytes;
      }
    }
  }
};

namespace {

using mhdgb::report_error;

size_t state_floats(int n) { return (size_t)2 * 6 * (n / 2 + 1) * (size_t)n * n; }

// Admission of one queued request: true when it left the queue (admitted, rejected or failed),
// false when it has to wait for memory.
bool admit(mhd_server_s& s, long long rid, Request& q) {
  const int n = q.r.n;
  const double L = q.r.L;
  int ci = s.free_class(n, L);
  if (ci < 0) {
    int cap = s.capacity_of(n);
    if (s.reserved + s.class_bytes(n, L, cap) > s.p.budget_bytes) s.reclaim();
    while (cap > 1 && s.reserved + s.class_bytes(n, L, cap) > s.p.budget_bytes) cap /= 2;  // a smaller class
    const double need = s.class_bytes(n, L, cap);
    if (s.reserved + need > s.p.budget_bytes) {
      if (s.class_bytes(n, L, 1) > s.p.budget_bytes) {
        q.status = MHD_REQ_REJECTED;
        q.code = MHD_ERR_OOM;
        q.error = "request does not fit the memory budget";
        return true;
      }
      return false;
    }
    const mhd_params prm = s.params_of(n, L);
    mhd_handle h = nullptr;
    if (mhd_batch_create(&prm, cap, &h) != MHD_OK) {
      q.status = MHD_REQ_REJECTED;
      q.code = MHD_ERR_OOM;
      q.error = std::string("size class allocation failed: ") + mhd_last_error();
      return true;
    }
    SizeClass c;
    c.h = h;
    c.n = n;
    c.L = L;
    c.cap = cap;
    c.bytes = need;
    ci = -1;
    for (size_t i = 0; i < s.classes.size(); ++i)
      if (!s.classes[i].h) { s.classes[i] = c; ci = (int)i; break; }
    if (ci < 0) { s.classes.push_back(c); ci = (int)s.classes.size() - 1; }
    s.reserved += need;
    if (s.reserved > s.peak) s.peak = s.reserved;
  }
  mhd_handle h = s.classes[ci].h;
  for (float v : q.init)
    if (!std::isfinite(v)) {
      q.status = MHD_REQ_FAILED;
      q.code = MHD_ERR_NONFINITE;
      q.error = "non-finite initial state";
      q.init.clear();
      return true;
    }
  const double dt = q.r.dt > 0 ? q.r.dt : 0.2 * q.r.L / n;
  int slot = -1, rc = mhd_batch_add(h, q.r.nu, q.r.eta, dt, &slot);
  if (rc == MHD_OK) rc = mhd_slot_set_state(h, slot, q.init.data());
  if (rc != MHD_OK) {
    if (slot >= 0) mhd_batch_remove(h, slot);
    q.status = MHD_REQ_FAILED;
    q.code = rc;
    q.error = mhd_last_error();
    q.init.clear();
    return true;
  }
  q.init.clear();
  q.init.shrink_to_fit();
  q.status = MHD_REQ_ACTIVE;
  q.cls = ci;
  q.slot = slot;
  s.active.push_back(rid);
  return true;
}

void retire(mhd_server_s& s, Request& q) {
  mhd_handle h = s.classes[q.cls].h;
  const int rc = mhd_slot_diagnostics(h, q.slot, q.diag, 8);
  if (rc != MHD_OK) {
    q.status = MHD_REQ_FAILED;
    q.code = rc;
    q.error = mhd_last_error();
  } else {
    q.status = MHD_REQ_DONE;
    if (s.p.keep_states) {
      q.result.resize(state_floats(q.r.n));
      if (mhd_slot_get_state(h, q.slot, q.result.data()) != MHD_OK) {
        q.status = MHD_REQ_FAILED;
        q.code = MHD_ERR_CUDA;
        q.error = mhd_last_error();
        q.result.clear();
      }
    }
  }
  mhd_batch_remove(h, q.slot);
  q.slot = -1;
}

}  // namespace

extern "C" {

int mhd_server_create(const mhd_server_params* params, mhd_server* out) {
  if (!params || !out) return report_error(MHD_ERR_INVALID, "null argument");
  *out = nullptr;
  if (!(params->budget_bytes > 0) || params->steps_per_tick < 1)
    return report_error(MHD_ERR_INVALID, "budget_bytes > 0 and steps_per_tick >= 1 required");
  if (params->scheme != MHD_RK4 && params->scheme != MHD_LSRK4)
    return report_error(MHD_ERR_INVALID, "scheme must be MHD_RK4 or MHD_LSRK4");
  for (int i = 0; i < 8; ++i)
    if (params->capacity[i] < 0) return report_error(MHD_ERR_INVALID, "capacities must be >= 0");
  mhd_server_s* s = new (std::nothrow) mhd_server_s();
  if (!s) return report_error(MHD_ERR_OOM, "host allocation failed");
  s->p = *params;
  *out = s;
  return MHD_OK;
}

int mhd_server_destroy(mhd_server s) {
  delete s;
  return MHD_OK;
}

int mhd_server_submit(mhd_server s, const mhd_request* req, long long* rid) {
  if (!s || !req || !rid) return report_error(MHD_ERR_INVALID, "null argument");
  if (!mhd_supported_n(req->n)) return report_error(MHD_ERR_INVALID, "unsupported grid size");
  if (!(req->L > 0) || !(req->nu >= 0) || !(req->eta >= 0) || req->steps < 1 || !std::isfinite(req->dt))
    return report_error(MHD_ERR_INVALID, "L > 0, nu, eta >= 0, finite dt and steps >= 1 required");
  Request q;
  q.r = *req;
  q.r.sol = nullptr;
  const size_t nf = state_floats(req->n);
  if (req->sol) q.init.assign(req->sol, req->sol + nf);
  else q.init.assign(nf, 0.f);
  const long long id = s->next++;
  s->reqs.emplace(id, std::move(q));
  s->queued.push_back(id);
  *rid = id;
  return MHD_OK;
}

int mhd_server_tick(mhd_server s, int* active, int* queued) {
  if (!s) return report_error(MHD_ERR_INVALID, "null server");
  // admission, first fit in arrival order
  for (size_t k = 0; k < s->queued.size();) {
    const long long id = s->queued[k];
    Request& q = s->reqs[id];
    if (q.status != MHD_REQ_QUEUED || admit(*s, id, q)) s->queued.erase(s->queued.begin() + k);
    else ++k;
  }
  if (!s->active.empty()) {
    long long nsteps = s->p.steps_per_tick;
    for (long long id : s->active) nsteps = std::min(nsteps, s->reqs[id].r.steps - s->reqs[id].done);
    std::vector<int> used;
    for (long long id : s->active) {
      const int c = s->reqs[id].cls;
      if (std::find(used.begin(), used.end(), c) == used.end()) used.push_back(c);
    }
    // every class steps on its own stream: launch all, then wait for all
    std::vector<int> bad;
    for (int c : used)
      if (mhd_step(s->classes[c].h, (int)nsteps) != MHD_OK) bad.push_back(c);
    for (int c : used)
      if (mhd_synchronize(s->classes[c].h) != MHD_OK && std::find(bad.begin(), bad.end(), c) == bad.end())
        bad.push_back(c);
    std::vector<long long> keep;
    for (long long id : s->active) {
      Request& q = s->reqs[id];
      if (std::find(bad.begin(), bad.end(), q.cls) != bad.end()) {
        q.status = MHD_REQ_FAILED;
        q.code = MHD_ERR_CUDA;
        q.error = "device error while stepping its size class";
        mhd_batch_remove(s->classes[q.cls].h, q.slot);
        continue;
      }
      q.done += nsteps;
      if (q.done >= q.r.steps) retire(*s, q);
      else keep.push_back(id);
    }
    s->active = keep;
  }
  if (active) *active = (int)s->active.size();
  if (queued) *queued = (int)s->queued.size();
  return MHD_OK;
}

int mhd_server_poll(mhd_server s, long long rid, int* status, long long* steps_done) {
  if (!s) return report_error(MHD_ERR_INVALID, "null server");
  auto it = s->reqs.find(rid);
  if (it == s->reqs.end()) return report_error(MHD_ERR_INVALID, "unknown request id");
  if (status) *status = it->second.status;
  if (steps_done) *steps_done = it->second.done;
  return MHD_OK;
}

int mhd_server_result(mhd_server s, long long rid, double* diag, float* sol) {
  if (!s) return report_error(MHD_ERR_INVALID, "null server");
  auto it = s->reqs.find(rid);
  if (it == s->reqs.end()) return report_error(MHD_ERR_INVALID, "unknown request id");
  const Request& q = it->second;
  if (q.status == MHD_REQ_FAILED || q.status == MHD_REQ_REJECTED) return report_error(q.code, q.error);
  if (q.status != MHD_REQ_DONE) return report_error(MHD_ERR_STATE, "request not finished");
  if (diag) std::memcpy(diag, q.diag, sizeof(q.diag));
  if (sol) {
    if (q.result.empty()) return report_error(MHD_ERR_STATE, "final states are kept only with keep_states");
    std::memcpy(sol, q.result.data(), q.result.size() * sizeof(float));
  }
  return MHD_OK;
}

int mhd_server_cancel(mhd_server s, long long rid) {
  if (!s) return report_error(MHD_ERR_INVALID, "null server");
  auto it = s->reqs.find(rid);
  if (it == s->reqs.end()) return report_error(MHD_ERR_INVALID, "unknown request id");
  Request& q = it->second;
  if (q.status == MHD_REQ_ACTIVE) {
    mhd_batch_remove(s->classes[q.cls].h, q.slot);
    s->active.erase(std::find(s->active.begin(), s->active.end(), rid));
  } else if (q.status == MHD_REQ_QUEUED) {
    s->queued.erase(std::find(s->queued.begin(), s->queued.end(), rid));
    q.init.clear();
  } else {
    return MHD_OK;  // already finished
  }
  q.status = MHD_REQ_CANCELLED;
  return MHD_OK;
}

int mhd_server_memory(mhd_server s, double* reserved, double* peak) {
  if (!s) return report_error(MHD_ERR_INVALID, "null server");
  if (reserved) *reserved = s->reserved;
  if (peak) *peak = s->peak;
  return MHD_OK;
}

}  // extern "C"
