// Serving loop: view-sessions with resident state, admitted against an HBM budget
// and a per-step pixel budget, whose queued frames are batched step by step.
//
// A session is admitted (its view allocated) in arrival order as soon as both
// budgets allow; it then keeps its reservoirs, AO and denoiser history and hash
// grid on the device across its frames. Each step takes the next queued frame of
// every admitted session and runs them as one vlt_batch_run on the server's stream;
// sessions that arrive or free their memory while steps are on the GPU join the
// next step. A closed session's view is freed once its queued and in-flight frames
// are done, which releases its budget for the waiting sessions.
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <deque>
#include <map>
#include <new>
#include <vector>

#include "vlt_internal.h"

using namespace vlt;

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct QFrame {
  vlt_frame_params fp;  // copied: the caller's may not outlive the call
  vlt_frame_inputs in;
  vlt_frame_outputs out;
  bool has_out;
  uint64_t tag;
  double t_submit;
};

struct Session {
  uint64_t id;
  uint32_t w, h;
  vlt_form form;
  vlt_params params;
  size_t bytes;
  vlt_view* view = nullptr;  // null while waiting
  std::deque<QFrame> queue;
  uint32_t in_flight = 0;
  bool closing = false;
  double t_open = 0, t_admit = 0;
};

struct StepRec {
  cudaEvent_t done;
  double t_issue;
  struct F {
    uint64_t session, tag;
    double t_submit;
  };
  std::vector<F> frames;
};

}  // namespace

struct vlt_server {
  vlt_ctx* ctx;
  vlt_server_config cfg;
  vlt_batch* batch = nullptr;
  uint64_t next_id = 1;
  std::map<uint64_t, Session> sessions;
  std::deque<uint64_t> waiting;  // arrival order
  std::deque<StepRec> in_flight;
  std::vector<cudaEvent_t> free_events;
  uint64_t bytes_in_use = 0, pixels_in_use = 0;
  uint32_t admitted = 0;
  vlt_server_stats stats;
};

namespace {

void admit(vlt_server* s) {
  while (!s->waiting.empty()) {
    auto it = s->sessions.find(s->waiting.front());
    if (it == s->sessions.end()) {
      s->waiting.pop_front();
      continue;
    }
    Session& se = it->second;
    const uint64_t px = (uint64_t)se.w * se.h;
    bool fits = s->bytes_in_use + se.bytes <= s->cfg.hbm_budget_bytes;
    if (s->cfg.step_pixel_budget && s->pixels_in_use + px > s->cfg.step_pixel_budget && s->admitted > 0)
      fits = false;
    if (s->cfg.max_sessions && s->admitted >= s->cfg.max_sessions) fits = false;
    if (!fits) break;  // strict arrival order
    vlt_view* v = nullptr;
    const vlt_status cst = vlt_view_create(s->ctx, se.w, se.h, se.form, &se.params, &v);
    if (cst != VLT_OK) {
      // The session keeps its place at the head of the queue and is tried again at
      // the next step, poll or close (a failed allocation leaves nothing behind).
      ++s->stats.admit_failures;
      s->stats.last_admit_status = (uint32_t)cst;
      break;
    }
    se.view = v;
    se.t_admit = now_ms();
    s->bytes_in_use += se.bytes;
    s->pixels_in_use += px;
    ++s->admitted;
    ++s->stats.sessions_admitted;
    s->stats.admit_wait_ms_total += se.t_admit - se.t_open;
    s->waiting.pop_front();
  }
}

void retire_closed(vlt_server* s) {
  for (auto it = s->sessions.begin(); it != s->sessions.end();) {
    Session& se = it->second;
    if (se.closing && se.queue.empty() && se.in_flight == 0) {
      if (se.view) {
        vlt_view_destroy(se.view);
        s->bytes_in_use -= se.bytes;
        s->pixels_in_use -= (uint64_t)se.w * se.h;
        --s->admitted;
      } else {
        for (auto w = s->waiting.begin(); w != s->waiting.end(); ++w)
          if (*w == se.id) {
            s->waiting.erase(w);
            break;
          }
      }
      ++s->stats.sessions_closed;
      it = s->sessions.erase(it);
    } else {
      ++it;
    }
  }
}

}  // namespace

extern "C" {

vlt_status vlt_server_create(vlt_ctx* ctx, const vlt_server_config* cfg, vlt_server** out) {
  if (!ctx || !cfg || !out || cfg->hbm_budget_bytes == 0) return VLT_ERR_INVALID_ARG;
  *out = nullptr;
  vlt_server* s = new (std::nothrow) vlt_server;
  if (!s) return VLT_ERR_OUT_OF_MEMORY;
  s->ctx = ctx;
  s->cfg = *cfg;
  memset(&s->stats, 0, sizeof(s->stats));
  vlt_status st = vlt_batch_create(ctx, &s->batch);
  if (st != VLT_OK) {
    delete s;
    return st;
  }
  *out = s;
  return VLT_OK;
}

vlt_status vlt_server_destroy(vlt_server* s) {
  if (!s) return VLT_OK;
  cudaSetDevice(ctx_device(s->ctx));
  for (StepRec& r : s->in_flight) {
    cudaEventSynchronize(r.done);
    cudaEventDestroy(r.done);
  }
  for (cudaEvent_t e : s->free_events) cudaEventDestroy(e);
  for (auto& kv : s->sessions)
    if (kv.second.view) vlt_view_destroy(kv.second.view);
  vlt_batch_destroy(s->batch);
  delete s;
  return VLT_OK;
}

vlt_batch* vlt_server_batch(vlt_server* s) { return s ? s->batch : nullptr; }

vlt_status vlt_server_open(vlt_server* s, uint32_t width, uint32_t height, vlt_form form, const vlt_params* params,
                           uint64_t* session) {
  if (!s || !params || !session || width == 0 || height == 0 || params->trace) return VLT_ERR_INVALID_ARG;
  size_t bytes = vlt_view_device_bytes(width, height, form, params);
  if (bytes == 0) return VLT_ERR_INVALID_ARG;
  if (bytes > s->cfg.hbm_budget_bytes) return VLT_ERR_BUDGET_EXCEEDED;  // could never be admitted
  Session se;
  se.id = s->next_id++;
  se.w = width;
  se.h = height;
  se.form = form;
  se.params = *params;
  se.bytes = bytes;
  se.t_open = now_ms();
  s->sessions.emplace(se.id, se);
  s->waiting.push_back(se.id);
  ++s->stats.sessions_opened;
  *session = se.id;
  return VLT_OK;
}

vlt_status vlt_server_submit(vlt_server* s, uint64_t session, const vlt_frame_inputs* in,
                             const vlt_frame_outputs* out, uint64_t tag) {
  if (!s || !in || !in->params) return VLT_ERR_INVALID_ARG;
  auto it = s->sessions.find(session);
  if (it == s->sessions.end() || it->second.closing) return VLT_ERR_BAD_STATE;
  QFrame f;
  f.fp = *in->params;
  f.in = *in;
  f.has_out = out != nullptr;
  if (out) f.out = *out;
  else memset(&f.out, 0, sizeof(f.out));
  f.tag = tag;
  f.t_submit = now_ms();
  it->second.queue.push_back(f);
  return VLT_OK;
}

vlt_status vlt_server_close(vlt_server* s, uint64_t session) {
  if (!s) return VLT_ERR_INVALID_ARG;
  auto it = s->sessions.find(session);
  if (it == s->sessions.end()) return VLT_ERR_BAD_STATE;
  it->second.closing = true;
  retire_closed(s);
  admit(s);
  return VLT_OK;
}

vlt_status vlt_server_step(vlt_server* s, void* stream, uint32_t* issued) {
  if (!s) return VLT_ERR_INVALID_ARG;
  if (issued) *issued = 0;
  vlt_status st = cuda_status(cudaSetDevice(ctx_device(s->ctx)));
  if (st != VLT_OK) return st;
  retire_closed(s);
  admit(s);
  std::vector<vlt_view*> views;
  std::vector<vlt_frame_inputs> ins;
  std::vector<vlt_frame_outputs> outs;
  std::vector<Session*> who;
  for (auto& kv : s->sessions) {
    Session& se = kv.second;
    if (!se.view || se.queue.empty()) continue;
    who.push_back(&se);
  }
  if (who.empty()) return VLT_OK;
  StepRec rec;
  rec.t_issue = now_ms();
  for (Session* se : who) {
    QFrame& f = se->queue.front();
    f.in.params = &f.fp;
    views.push_back(se->view);
    ins.push_back(f.in);
    outs.push_back(f.out);
    rec.frames.push_back({se->id, f.tag, f.t_submit});
  }
  st = vlt_batch_run(s->batch, views.data(), ins.data(), outs.data(), (uint32_t)views.size(), stream);
  if (st != VLT_OK) return st;
  if (s->free_events.empty()) {
    cudaEvent_t e;
    st = cuda_status(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (st != VLT_OK) return st;
    s->free_events.push_back(e);
  }
  rec.done = s->free_events.back();
  s->free_events.pop_back();
  st = cuda_status(cudaEventRecord(rec.done, (cudaStream_t)stream));
  if (st != VLT_OK) return st;
  uint64_t px = 0;
  for (Session* se : who) {
    se->queue.pop_front();
    ++se->in_flight;
    px += (uint64_t)se->w * se->h;
  }
  s->in_flight.push_back(std::move(rec));
  ++s->stats.steps;
  s->stats.frames_issued += who.size();
  s->stats.pixels_issued += px;
  if (issued) *issued = (uint32_t)who.size();
  return VLT_OK;
}

uint32_t vlt_server_poll(vlt_server* s, vlt_server_completion* out, uint32_t max, int wait) {
  if (!s) return 0;
  cudaSetDevice(ctx_device(s->ctx));
  uint32_t k = 0;
  bool waited = false;
  while (!s->in_flight.empty()) {
    StepRec& r = s->in_flight.front();
    if (out && k + r.frames.size() > max) break;
    cudaError_t q = cudaEventQuery(r.done);
    if (q == cudaErrorNotReady) {
      if (!wait || waited) break;
      cudaEventSynchronize(r.done);
      waited = true;
    } else if (q != cudaSuccess) {
      cudaGetLastError();
    }
    double t = now_ms();
    for (const StepRec::F& f : r.frames) {
      if (out) {
        out[k].session = f.session;
        out[k].tag = f.tag;
        out[k].latency_ms = t - f.t_submit;
        out[k].step_ms = t - r.t_issue;
      }
      ++k;
      auto it = s->sessions.find(f.session);
      if (it != s->sessions.end() && it->second.in_flight) --it->second.in_flight;
      ++s->stats.frames_done;
    }
    s->free_events.push_back(r.done);
    s->in_flight.pop_front();
  }
  retire_closed(s);
  admit(s);
  return k;
}

vlt_status vlt_server_get_stats(const vlt_server* s, vlt_server_stats* out) {
  if (!s || !out) return VLT_ERR_INVALID_ARG;
  *out = s->stats;
  out->sessions_live = s->admitted;
  out->sessions_waiting = (uint32_t)s->waiting.size();
  out->bytes_in_use = s->bytes_in_use;
  out->pixels_in_use = s->pixels_in_use;
  out->steps_in_flight = (uint32_t)s->in_flight.size();
  return VLT_OK;
}

}  // extern "C"
