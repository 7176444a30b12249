// Batched frames: one frame of many views as one stream of batched launches.
//
// Each view's frame driver runs in recording mode (every launch becomes a Job with
// its parameter tuple). The executor then repeatedly takes the next job of every
// view, picks the kernel that most views run next, and turns those views' jobs into
// one persistent k_batched launch over their concatenated tile lists. Jobs of one
// view stay in order (they are dependent); jobs of different views are independent,
// so grouping them changes no result. All tile maps and parameter tuples of the
// step go into one argument arena (pinned host memory, double-buffered), copied to
// the device with one cudaMemcpyAsync ahead of the kernels; the step is captured in
// a CUDA graph, cached under the signature of its launch sequence, and replayed on
// later steps with the same sequence (only the arena's contents change).
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "vlt_internal.h"

using namespace vlt;

namespace {

struct Arena {
  uint8_t* host = nullptr;
  uint8_t* dev = nullptr;
  size_t cap = 0;
  cudaEvent_t copied = nullptr;  // recorded after the step's upload from this arena
  bool pending = false;
};

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  uint64_t last_use = 0;
};

const TileShape kCandidates[VLT_TILE_CANDIDATES] = {{32, 4}, {16, 8}, {32, 8}, {16, 16}, {64, 4}};

struct TuneRec {
  std::string name;
  double ns[VLT_TILE_CANDIDATES] = {0, 0, 0, 0, 0};
  double kpix[VLT_TILE_CANDIDATES] = {0, 0, 0, 0, 0};
  int chosen = 0;
};

}  // namespace

struct vlt_batch {
  vlt_ctx* ctx;
  Arena arena[2];
  int parity = 0;
  bool graphs = true;
  std::unordered_map<std::string, GraphEntry> cache;
  uint64_t tick = 0;
  std::map<const void*, TileShape> shapes;  // per kernel (PrepareFn) chosen tile shape
  // autotuner
  int tune_left = 0;   // frames still to run while tuning
  int tune_index = 0;  // frames run while tuning
  std::map<const void*, TuneRec> tune;
  std::vector<cudaEvent_t> events;
  vlt_batch_stats stats;
};

namespace {

const size_t kMaxGraphs = 32;

vlt_status ensure_arena(Arena& a, size_t bytes) {
  if (a.cap >= bytes) return VLT_OK;
  if (a.pending) {
    cudaEventSynchronize(a.copied);
    a.pending = false;
  }
  if (a.host) cudaFreeHost(a.host);
  if (a.dev) cudaFree(a.dev);
  a.host = nullptr;
  a.dev = nullptr;
  a.cap = 0;
  size_t cap = 1 << 16;
  while (cap < bytes) cap <<= 1;
  vlt_status st = cuda_status(cudaHostAlloc((void**)&a.host, cap, cudaHostAllocDefault));
  if (st != VLT_OK) return st;
  st = cuda_status(cudaMalloc((void**)&a.dev, cap));
  if (st != VLT_OK) {
    cudaFreeHost(a.host);
    a.host = nullptr;
    return st;
  }
  if (!a.copied) {
    st = cuda_status(cudaEventCreateWithFlags(&a.copied, cudaEventDisableTiming));
    if (st != VLT_OK) return st;
  }
  a.cap = cap;
  return VLT_OK;
}

// Grouping of the recorded jobs into batched launches (see the file comment).
struct Group {
  PrepareFn key;
  std::vector<const Job*> jobs;
};

std::vector<Group> group_jobs(const std::vector<Recorder>& recs) {
  std::vector<Group> groups;
  std::vector<size_t> head(recs.size(), 0);
  for (;;) {
    // Count heads per kernel; pick the most common (first seen on ties).
    std::vector<std::pair<PrepareFn, uint32_t>> counts;
    for (size_t k = 0; k < recs.size(); ++k) {
      if (head[k] >= recs[k].jobs.size()) continue;
      PrepareFn f = recs[k].jobs[head[k]].prepare;
      bool found = false;
      for (auto& c : counts)
        if (c.first == f) {
          ++c.second;
          found = true;
          break;
        }
      if (!found) counts.push_back({f, 1u});
    }
    if (counts.empty()) break;
    PrepareFn best = counts[0].first;
    uint32_t bc = counts[0].second;
    for (auto& c : counts)
      if (c.second > bc) {
        best = c.first;
        bc = c.second;
      }
    Group g;
    g.key = best;
    for (size_t k = 0; k < recs.size(); ++k) {
      if (head[k] >= recs[k].jobs.size()) continue;
      const Job& j = recs[k].jobs[head[k]];
      if (j.prepare != best) continue;
      g.jobs.push_back(&j);
      ++head[k];
    }
    groups.push_back(std::move(g));
  }
  return groups;
}

TileShape shape_for(vlt_batch* b, const Job& j) {
  if (j.one_d) return TileShape();
  if (b->tune_left > 0) return kCandidates[b->tune_index % VLT_TILE_CANDIDATES];
  auto it = b->shapes.find((const void*)j.prepare);
  return it == b->shapes.end() ? TileShape() : it->second;
}

void finish_tuning(vlt_batch* b) {
  for (auto& kv : b->tune) {
    TuneRec& t = kv.second;
    int best = -1;
    double best_v = 0;
    for (int c = 0; c < VLT_TILE_CANDIDATES; ++c) {
      if (t.kpix[c] <= 0) continue;
      double v = t.ns[c] / t.kpix[c];
      if (best < 0 || v < best_v) {
        best = c;
        best_v = v;
      }
    }
    if (best >= 0) {
      t.chosen = best;
      b->shapes[kv.first] = kCandidates[best];
    }
  }
}

}  // namespace

extern "C" {

vlt_status vlt_batch_create(vlt_ctx* ctx, vlt_batch** out) {
  if (!ctx || !out) return VLT_ERR_INVALID_ARG;
  *out = nullptr;
  vlt_status st = cuda_status(cudaSetDevice(ctx_device(ctx)));
  if (st != VLT_OK) return st;
  vlt_batch* b = new (std::nothrow) vlt_batch;
  if (!b) return VLT_ERR_OUT_OF_MEMORY;
  b->ctx = ctx;
  memset(&b->stats, 0, sizeof(b->stats));
  *out = b;
  return VLT_OK;
}

vlt_status vlt_batch_destroy(vlt_batch* b) {
  if (!b) return VLT_OK;
  cudaSetDevice(ctx_device(b->ctx));
  for (auto& a : b->arena) {
    if (a.pending) cudaEventSynchronize(a.copied);
    if (a.copied) cudaEventDestroy(a.copied);
    if (a.host) cudaFreeHost(a.host);
    if (a.dev) cudaFree(a.dev);
  }
  for (auto& kv : b->cache) cudaGraphExecDestroy(kv.second.exec);
  for (cudaEvent_t e : b->events) cudaEventDestroy(e);
  delete b;
  return VLT_OK;
}

vlt_status vlt_batch_set_graphs(vlt_batch* b, int enable) {
  if (!b) return VLT_ERR_INVALID_ARG;
  b->graphs = enable != 0;
  return VLT_OK;
}

vlt_status vlt_batch_autotune(vlt_batch* b) {
  if (!b) return VLT_ERR_INVALID_ARG;
  b->tune.clear();
  b->tune_index = 0;
  b->tune_left = 2 * VLT_TILE_CANDIDATES;
  return VLT_OK;
}

uint32_t vlt_batch_tile_table(const vlt_batch* b, vlt_tile_choice* out, uint32_t max) {
  if (!b) return 0;
  uint32_t k = 0;
  for (const auto& kv : b->tune) {
    if (out && k < max) {
      vlt_tile_choice& c = out[k];
      memset(&c, 0, sizeof(c));
      strncpy(c.pass, kv.second.name.c_str(), sizeof(c.pass) - 1);
      auto it = b->shapes.find(kv.first);
      TileShape s = it == b->shapes.end() ? TileShape() : it->second;
      c.bx = s.bx;
      c.by = s.by;
      for (int i = 0; i < VLT_TILE_CANDIDATES; ++i)
        c.ns_per_kpix[i] = kv.second.kpix[i] > 0 ? (float)(kv.second.ns[i] / kv.second.kpix[i]) : 0.0f;
    }
    ++k;
  }
  return k;
}

vlt_status vlt_batch_get_stats(const vlt_batch* b, vlt_batch_stats* out) {
  if (!b || !out) return VLT_ERR_INVALID_ARG;
  *out = b->stats;
  return VLT_OK;
}

vlt_status vlt_batch_run(vlt_batch* b, vlt_view* const* views, const vlt_frame_inputs* inputs,
                         const vlt_frame_outputs* outputs, uint32_t n, void* stream) {
  if (!b || (n && (!views || !inputs))) return VLT_ERR_INVALID_ARG;
  if (n == 0) return VLT_OK;
  const int dev = ctx_device(b->ctx);
  for (uint32_t k = 0; k < n; ++k) {
    if (!views[k] || view_device(views[k]) != dev || !frame_inputs_ok(views[k], &inputs[k]))
      return VLT_ERR_INVALID_ARG;
    for (uint32_t j = 0; j < k; ++j)
      if (views[j] == views[k]) return VLT_ERR_INVALID_ARG;
  }
  vlt_status st = cuda_status(cudaSetDevice(dev));
  if (st != VLT_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;

  // 1. Record every view's frame.
  std::vector<Recorder> recs(n);
  uint32_t jobs = 0;
  for (uint32_t k = 0; k < n; ++k) {
    st = record_frame(views[k], &inputs[k], outputs ? &outputs[k] : nullptr, &recs[k]);
    if (st != VLT_OK) return st;
    jobs += (uint32_t)recs[k].jobs.size();
  }

  // 2. Group and prepare into the argument arena.
  std::vector<Group> groups = group_jobs(recs);
  const bool tuning = b->tune_left > 0;
  Arena& a = b->arena[b->parity];
  if (a.pending) {  // the upload two steps ago must be done before the host arena is rewritten
    cudaEventSynchronize(a.copied);
    a.pending = false;
  }
  std::vector<Prepared> preps(groups.size());
  size_t used = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    used = 0;
    bool fits = true;
    for (size_t g = 0; g < groups.size(); ++g) {
      const Job& j0 = *groups[g].jobs[0];
      // worst-case size: tile map + tuples, 16-byte aligned
      size_t need = (2 * groups[g].jobs.size() + 1) * 4 + 16 + groups[g].jobs.size() * (j0.args.size() + 16) + 16;
      if (used + need > a.cap) {
        fits = false;
        used += need;
        continue;
      }
      used += groups[g].key(groups[g].jobs.data(), (uint32_t)groups[g].jobs.size(), shape_for(b, j0), a.host, used,
                            &preps[g]);
    }
    if (fits) break;
    // A new arena invalidates every captured graph (their copy and kernel nodes
    // hold the old addresses).
    for (auto& kv : b->cache) cudaGraphExecDestroy(kv.second.exec);
    b->cache.clear();
    st = ensure_arena(a, used + (1 << 12));
    if (st != VLT_OK) return st;
  }
  for (Prepared& p : preps) p.dev_base = a.dev;

  // 3. Issue: the upload, then the launches (from a cached graph when possible).
  // The legacy default stream cannot be captured: steps on it are issued directly.
  const bool use_graph = b->graphs && !tuning && s != 0;
  std::string sig;
  if (use_graph) {
    sig.reserve(groups.size() * 40 + 16);
    char buf[96];
    snprintf(buf, sizeof(buf), "%d:%zu:%p;", b->parity, used, (void*)a.dev);
    sig += buf;
    for (const Prepared& p : preps) {
      snprintf(buf, sizeof(buf), "%p,%u,%u,%u,%u,%u,%zu;", p.key, p.n_jobs, p.total_tiles, p.grid, p.block.x,
               p.block.y, p.arena_off);
      sig += buf;
    }
  }
  auto issue = [&](bool timed) -> vlt_status {
    vlt_status e = cuda_status(cudaMemcpyAsync(a.dev, a.host, used, cudaMemcpyHostToDevice, s));
    if (e != VLT_OK) return e;
    for (size_t g = 0; g < preps.size(); ++g) {
      if (timed) cudaEventRecord(b->events[2 * g], s);
      preps[g].launch(preps[g], s);
      if (timed) cudaEventRecord(b->events[2 * g + 1], s);
    }
    return cuda_status(cudaGetLastError());
  };
  if (tuning) {
    while (b->events.size() < 2 * preps.size()) {
      cudaEvent_t e;
      st = cuda_status(cudaEventCreate(&e));
      if (st != VLT_OK) return st;
      b->events.push_back(e);
    }
    st = issue(true);
    if (st != VLT_OK) return st;
    st = cuda_status(cudaEventRecord(a.copied, s));
    if (st != VLT_OK) return st;
    st = cuda_status(cudaStreamSynchronize(s));
    if (st != VLT_OK) return st;
    const int cand = b->tune_index % VLT_TILE_CANDIDATES;
    for (size_t g = 0; g < preps.size(); ++g) {
      const Job& j0 = *groups[g].jobs[0];
      if (j0.one_d) continue;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, b->events[2 * g], b->events[2 * g + 1]);
      double kpix = 0;
      for (const Job* j : groups[g].jobs) kpix += (double)j->w * j->h / 1e3;
      TuneRec& t = b->tune[(const void*)groups[g].key];
      if (t.name.empty()) t.name = j0.name;
      t.ns[cand] += ms * 1e6;
      t.kpix[cand] += kpix;
    }
    ++b->tune_index;
    if (--b->tune_left == 0) finish_tuning(b);
  } else if (use_graph) {
    auto it = b->cache.find(sig);
    if (it == b->cache.end()) {
      if (b->cache.size() >= kMaxGraphs) {  // evict the least recently used
        auto victim = b->cache.begin();
        for (auto c = b->cache.begin(); c != b->cache.end(); ++c)
          if (c->second.last_use < victim->second.last_use) victim = c;
        cudaGraphExecDestroy(victim->second.exec);
        b->cache.erase(victim);
      }
      cudaGraph_t graph = nullptr;
      st = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      if (st != VLT_OK) return st;
      vlt_status ist = issue(false);
      cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (ist != VLT_OK) {
        if (graph) cudaGraphDestroy(graph);
        return ist;
      }
      st = cuda_status(ce);
      if (st != VLT_OK) return st;
      GraphEntry ge;
      st = cuda_status(cudaGraphInstantiate(&ge.exec, graph, 0));
      cudaGraphDestroy(graph);
      if (st != VLT_OK) return st;
      it = b->cache.emplace(sig, ge).first;
      ++b->stats.graph_captures;
    } else {
      ++b->stats.graph_replays;
    }
    it->second.last_use = ++b->tick;
    st = cuda_status(cudaGraphLaunch(it->second.exec, s));
    if (st != VLT_OK) return st;
    st = cuda_status(cudaEventRecord(a.copied, s));
    if (st != VLT_OK) return st;
  } else {
    st = issue(false);
    if (st != VLT_OK) return st;
    st = cuda_status(cudaEventRecord(a.copied, s));
    if (st != VLT_OK) return st;
  }
  a.pending = true;
  b->parity ^= 1;
  ++b->stats.frames;
  b->stats.launches += preps.size();
  b->stats.last_launches = (uint32_t)preps.size();
  b->stats.last_jobs = jobs;
  b->stats.arena_bytes = used;
  return VLT_OK;
}

}  // extern "C"
