// Batched frames: one frame of many views as one stream of batched launches.
//
// Each view's frame driver runs in recording mode (every launch becomes a Job with
// its parameter tuple). The executor then repeatedly takes the next job of every
// view, picks the kernel that most views run next, and turns those views' jobs into
// one persistent k_batched launch over their concatenated tile lists, with the
// views' parameter tuples and tile map in the kernel's parameter block. Jobs of one
// view stay in order (they are dependent); jobs of different views are independent,
// so grouping them changes no result. A recorded frame tags its jobs with a lane
// (main, hash grid, specular, AO) and marks where the side lanes fork and join; the
// executor groups each lane separately and issues the side lanes on its own streams
// between the fork and the joins, as a single view's frame does. With graphs on,
// the step's launches are
// captured into a CUDA graph; a cached executable graph with the same launch
// sequence is updated in place with the new parameters (cudaGraphExecUpdate) and
// replayed, otherwise a new one is instantiated.
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

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  uint64_t last_use = 0;
};

// Candidate launch shapes: five tile shapes, each one tile per block and persistent.
const TileShape kCandidates[VLT_TILE_CANDIDATES] = {{32, 4, 0}, {16, 8, 0}, {32, 8, 0}, {16, 16, 0}, {64, 4, 0},
                                                    {32, 4, 1}, {16, 8, 1}, {32, 8, 1}, {16, 16, 1}, {64, 4, 1}};

struct TuneRec {
  std::string name;
  double ns[VLT_TILE_CANDIDATES] = {};
  double kpix[VLT_TILE_CANDIDATES] = {};
  int chosen = 0;
};

}  // namespace

struct vlt_batch {
  vlt_ctx* ctx;
  std::vector<uint8_t> params;  // parameter blocks of the step being issued
  bool graphs = true;
  uint64_t chunk_pixels = ~(uint64_t)0;  // no chunking
  bool persistent = false;
  std::unordered_map<std::string, GraphEntry> cache;
  uint64_t tick = 0;
  std::map<const void*, TileShape> shapes;  // per kernel (PrepareFn) chosen tile shape
  // autotuner
  int tune_left = 0;   // frames still to run while tuning
  int tune_index = 0;  // frames run while tuning
  std::map<const void*, TuneRec> tune;
  std::vector<cudaEvent_t> events;
  vlt_batch_stats stats;
  // side streams of the lanes (kLanes) and their fork/join events
  cudaStream_t lane_stream[kLanes] = {};
  cudaEvent_t fork_event = nullptr;
  cudaEvent_t join_event[kLanes] = {};
  bool lanes_ok = false;
};

namespace {

const size_t kMaxGraphs = 32;

// Grouping of the recorded jobs into batched launches (see the file comment).
struct Group {
  PrepareFn key;       // null: a stream marker
  uint8_t marker = 0;
  uint8_t lane = 0;
  std::vector<const Job*> jobs;
};

// One lane of the recorded frames: its jobs in order (lane 0 keeps the markers).
struct LaneList {
  std::vector<const Job*> jobs;
};

std::vector<Group> group_jobs(const std::vector<LaneList>& lists, uint8_t lane) {
  std::vector<Group> groups;
  std::vector<size_t> head(lists.size(), 0);
  auto same = [](const Job* a, const Job* c) { return a->prepare == c->prepare && a->marker == c->marker; };
  for (;;) {
    // Count heads per kernel (or marker); pick the most common (first seen on ties).
    std::vector<std::pair<const Job*, uint32_t>> counts;
    for (size_t k = 0; k < lists.size(); ++k) {
      if (head[k] >= lists[k].jobs.size()) continue;
      const Job* f = lists[k].jobs[head[k]];
      bool found = false;
      for (auto& c : counts)
        if (same(c.first, f)) {
          ++c.second;
          found = true;
          break;
        }
      if (!found) counts.push_back({f, 1u});
    }
    if (counts.empty()) break;
    const Job* best = counts[0].first;
    uint32_t bc = counts[0].second;
    for (auto& c : counts)
      if (c.second > bc) {
        best = c.first;
        bc = c.second;
      }
    Group g;
    g.key = best->prepare;
    g.marker = best->marker;
    g.lane = lane;
    for (size_t k = 0; k < lists.size(); ++k) {
      if (head[k] >= lists[k].jobs.size()) continue;
      const Job* j = lists[k].jobs[head[k]];
      if (!same(j, best)) continue;
      g.jobs.push_back(j);
      ++head[k];
    }
    groups.push_back(std::move(g));
  }
  return groups;
}

// The groups of one chunk of views in issue order: the main lane up to the fork
// marker, then every side lane's groups, then the rest of the main lane (with its
// join markers).
std::vector<Group> order_chunk(const std::vector<const Recorder*>& recs) {
  std::vector<LaneList> lists[kLanes + 1];
  for (int l = 0; l <= kLanes; ++l) lists[l].resize(recs.size());
  for (size_t k = 0; k < recs.size(); ++k)
    for (const Job& j : recs[k]->jobs) lists[j.prepare ? j.lane : 0][k].jobs.push_back(&j);
  std::vector<Group> main = group_jobs(lists[0], 0);
  std::vector<Group> out;
  size_t i = 0;
  bool forked = false;
  for (; i < main.size() && !forked; ++i) {
    forked = !main[i].key && main[i].marker == kMarkFork;
    out.push_back(std::move(main[i]));
  }
  for (int l = 1; l <= kLanes; ++l) {
    std::vector<Group> g = group_jobs(lists[l], (uint8_t)l);
    for (Group& x : g) out.push_back(std::move(x));
  }
  for (; i < main.size(); ++i) out.push_back(std::move(main[i]));
  return out;
}

TileShape shape_for(vlt_batch* b, const Job& j) {
  if (!j.one_d) {
    if (b->tune_left > 0) return kCandidates[b->tune_index % VLT_TILE_CANDIDATES];
    auto it = b->shapes.find((const void*)j.prepare);
    if (it != b->shapes.end()) return it->second;
  }
  TileShape t;
  t.persistent = b->persistent ? 1 : 0;
  return t;
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
  b->lanes_ok = cudaEventCreateWithFlags(&b->fork_event, cudaEventDisableTiming) == cudaSuccess;
  for (int l = 0; l < kLanes; ++l) {
    if (cudaStreamCreateWithFlags(&b->lane_stream[l], cudaStreamNonBlocking) != cudaSuccess) b->lanes_ok = false;
    if (cudaEventCreateWithFlags(&b->join_event[l], cudaEventDisableTiming) != cudaSuccess) b->lanes_ok = false;
  }
  (void)cudaGetLastError();  // without side streams every lane runs on the step's stream
  *out = b;
  return VLT_OK;
}

vlt_status vlt_batch_destroy(vlt_batch* b) {
  if (!b) return VLT_OK;
  cudaSetDevice(ctx_device(b->ctx));
  for (auto& kv : b->cache) cudaGraphExecDestroy(kv.second.exec);
  for (cudaEvent_t e : b->events) cudaEventDestroy(e);
  for (int l = 0; l < kLanes; ++l) {
    if (b->lane_stream[l]) cudaStreamDestroy(b->lane_stream[l]);
    if (b->join_event[l]) cudaEventDestroy(b->join_event[l]);
  }
  if (b->fork_event) cudaEventDestroy(b->fork_event);
  delete b;
  return VLT_OK;
}

vlt_status vlt_batch_set_graphs(vlt_batch* b, int enable) {
  if (!b) return VLT_ERR_INVALID_ARG;
  b->graphs = enable != 0;
  return VLT_OK;
}

vlt_status vlt_batch_set_chunk_pixels(vlt_batch* b, uint64_t pixels) {
  if (!b || pixels == 0) return VLT_ERR_INVALID_ARG;
  b->chunk_pixels = pixels;
  return VLT_OK;
}

vlt_status vlt_batch_set_persistent(vlt_batch* b, int enable) {
  if (!b) return VLT_ERR_INVALID_ARG;
  b->persistent = enable != 0;
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
      c.persistent = s.persistent;
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
    if (!views[k] || view_device(views[k]) != dev || view_traced(views[k]) || !frame_inputs_ok(views[k], &inputs[k]) ||
        !frame_outputs_ok(views[k], outputs ? &outputs[k] : nullptr))
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

  // 2. Pack the views into chunks of at most chunk_pixels (first fit, largest
  // first; a larger view is a chunk of its own). A chunk's whole frame runs before
  // the next chunk's, so what one pass writes is still in L2 when the next pass of
  // the same views reads it. Then group each chunk's jobs into batched launches.
  std::vector<uint32_t> order(n);
  for (uint32_t k = 0; k < n; ++k) order[k] = k;
  auto px = [&](uint32_t k) { return (uint64_t)view_width(views[k]) * view_height(views[k]); };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return px(a) > px(c); });
  std::vector<std::vector<uint32_t>> chunks;
  std::vector<uint64_t> fill;
  for (uint32_t k : order) {
    size_t c = 0;
    while (c < chunks.size() && fill[c] + px(k) > b->chunk_pixels) ++c;
    if (c == chunks.size()) {
      chunks.emplace_back();
      fill.push_back(0);
    }
    chunks[c].push_back(k);
    fill[c] += px(k);
  }
  std::vector<Group> groups;
  for (const auto& ch : chunks) {
    std::vector<const Recorder*> rs;
    for (uint32_t k : ch) rs.push_back(&recs[k]);
    std::vector<Group> g = order_chunk(rs);
    for (Group& x : g) groups.push_back(std::move(x));
  }
  b->stats.last_chunks = (uint32_t)chunks.size();
  const bool tuning = b->tune_left > 0;
  b->params.clear();
  std::vector<Prepared> preps;
  std::vector<size_t> group_of;  // prepared launch -> group
  // The step as a list of operations: a prepared launch (>= 0) or a stream marker
  // (-1 - marker).
  std::vector<long> ops;
  for (size_t g = 0; g < groups.size(); ++g) {
    if (!groups[g].key) {
      ops.push_back(-1 - (long)groups[g].marker);
      continue;
    }
    size_t before = preps.size();
    groups[g].key(groups[g].jobs.data(), (uint32_t)groups[g].jobs.size(), shape_for(b, *groups[g].jobs[0]),
                  b->params, preps);
    for (size_t k = before; k < preps.size(); ++k) {
      group_of.push_back(g);
      ops.push_back((long)k);
    }
  }
  const uint8_t* params = b->params.data();

  // 3. Issue the launches (through a CUDA graph when possible).
  // The legacy default stream cannot be captured: steps on it are issued directly.
  const bool use_graph = b->graphs && !tuning && s != 0;
  // Side lanes run on their own streams (forked from s after the fork marker, joined
  // back at their join markers and at the end); timed (tuning) steps run on s alone.
  auto issue = [&](bool timed) -> vlt_status {
    const bool use_lanes = !timed && b->lanes_ok;
    bool forked = false, joined[kLanes + 1] = {};
    auto join = [&](int l) {
      if (!forked || joined[l]) return;
      cudaEventRecord(b->join_event[l - 1], b->lane_stream[l - 1]);
      cudaStreamWaitEvent(s, b->join_event[l - 1], 0);
      joined[l] = true;
    };
    for (long op : ops) {
      if (op < 0) {
        const int m = (int)(-1 - op);
        if (!use_lanes) continue;
        if (m == kMarkFork) {
          if (forked)
            for (int l = 1; l <= kLanes; ++l) join(l);  // a chunk's second fork
          cudaEventRecord(b->fork_event, s);
          for (int l = 1; l <= kLanes; ++l) {
            cudaStreamWaitEvent(b->lane_stream[l - 1], b->fork_event, 0);
            joined[l] = false;
          }
          forked = true;
        } else if (m > kMarkJoin && m <= kMarkJoin + kLanes) {
          join(m - kMarkJoin);
        }
        continue;
      }
      const size_t k = (size_t)op;
      const int lane = groups[group_of[k]].lane;
      cudaStream_t ls = (use_lanes && forked && lane > 0) ? b->lane_stream[lane - 1] : s;
      if (timed) cudaEventRecord(b->events[2 * k], s);
      preps[k].launch(preps[k], params, ls);
      if (timed) cudaEventRecord(b->events[2 * k + 1], s);
    }
    if (use_lanes)
      for (int l = 1; l <= kLanes; ++l) join(l);
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
    st = cuda_status(cudaStreamSynchronize(s));
    if (st != VLT_OK) return st;
    const int cand = b->tune_index % VLT_TILE_CANDIDATES;
    for (size_t k = 0; k < preps.size(); ++k) {
      const Group& gr = groups[group_of[k]];
      const Job& j0 = *gr.jobs[0];
      if (j0.one_d) continue;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, b->events[2 * k], b->events[2 * k + 1]);
      TuneRec& t = b->tune[(const void*)gr.key];
      if (t.name.empty()) t.name = j0.name;
      t.ns[cand] += ms * 1e6;
    }
    for (const Group& gr : groups) {
      if (!gr.key || gr.jobs[0]->one_d) continue;
      double kpix = 0;
      for (const Job* j : gr.jobs) kpix += (double)j->w * j->h / 1e3;
      b->tune[(const void*)gr.key].kpix[cand] += kpix;
    }
    ++b->tune_index;
    if (--b->tune_left == 0) finish_tuning(b);
  } else if (use_graph) {
    std::string sig;
    sig.reserve(preps.size() * 48);
    char buf[96];
    for (long op : ops) {
      if (op < 0) {
        snprintf(buf, sizeof(buf), "m%ld;", -1 - op);
      } else {
        const Prepared& p = preps[(size_t)op];
        snprintf(buf, sizeof(buf), "%p,%u,%u,%u,%zu,%u;", p.key, p.grid, p.block.x, p.block.y, p.param_bytes,
                 (unsigned)groups[group_of[(size_t)op]].lane);
      }
      sig += buf;
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
    auto it = b->cache.find(sig);
    bool updated = false;
    if (it != b->cache.end()) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(it->second.exec, graph, &info) == cudaSuccess) {
        updated = true;
        ++b->stats.graph_replays;
      } else {
        cudaGetLastError();
        cudaGraphExecDestroy(it->second.exec);
        b->cache.erase(it);
        it = b->cache.end();
      }
    }
    if (!updated) {
      if (b->cache.size() >= kMaxGraphs) {  // evict the least recently used
        auto victim = b->cache.begin();
        for (auto c = b->cache.begin(); c != b->cache.end(); ++c)
          if (c->second.last_use < victim->second.last_use) victim = c;
        cudaGraphExecDestroy(victim->second.exec);
        b->cache.erase(victim);
      }
      GraphEntry ge;
      st = cuda_status(cudaGraphInstantiate(&ge.exec, graph, 0));
      if (st != VLT_OK) {
        cudaGraphDestroy(graph);
        return st;
      }
      it = b->cache.emplace(sig, ge).first;
      ++b->stats.graph_captures;
    }
    cudaGraphDestroy(graph);
    it->second.last_use = ++b->tick;
    st = cuda_status(cudaGraphLaunch(it->second.exec, s));
    if (st != VLT_OK) return st;
  } else {
    st = issue(false);
    if (st != VLT_OK) return st;
  }
  ++b->stats.frames;
  b->stats.launches += preps.size();
  b->stats.last_launches = (uint32_t)preps.size();
  b->stats.last_jobs = jobs;
  b->stats.arena_bytes = b->params.size();
  return VLT_OK;
}

}  // extern "C"
