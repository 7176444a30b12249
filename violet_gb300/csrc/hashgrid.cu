// Spatial-hash-grid radiance cache: per-bucket decay/compaction, query emission,
// deterministic cell insertion + random per-cell query selection, compaction of
// the selected queries, and the cell radiance update.
//
// Insertion order. The shader inserts cells with InterlockedCompareExchange, so
// which of several racing new cells gets which slot depends on timing. Here the
// result is defined as if the queries were processed one at a time in query-index
// order (the CPU restatement does exactly that), and the GPU reproduces it:
//   S1  every query probes its bucket; a hit selects immediately (atomicMax is
//       order-independent); a miss with a free slot is counted per bucket and
//       sets its bit in a miss bitmask;
//   S2  each bucket with misses gets a contiguous segment of a miss list and is
//       listed among the buckets with misses;
//   S3  the misses (the bitmask's bits) are scattered into their bucket's segment
//       (any order);
//   S4  one warp per listed bucket repeatedly takes the smallest unresolved query
//       index, probes/inserts its checksum exactly as the sequential loop would,
//       and resolves every listed query with that checksum.
#include <mutex>

#include "hashgrid.cuh"
#include "vlt_compact.cuh"
#include "vlt_internal.h"

namespace vlt {

// --------------------------------------------------------------- emission

// V8: the query buffer is 32-byte aligned and each record is written with one
// 256-bit store (the frame driver's buffers always are; the per-pass entry point
// checks the caller's pointer).
template <bool V8>
struct HgEmitF {
  static __device__ __forceinline__ void store(uint32_t* __restrict__ queries, uint32_t q, uint4 a, uint4 b) {
    if (V8) {
      st_rec32(queries + (size_t)q * Q_WORDS, a, b);
    } else {
      uint4* rec = (uint4*)(queries + (size_t)q * Q_WORDS);
      rec[0] = a;
      rec[1] = b;
    }
  }
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, uint32_t bucket_mask, uint32_t key_mode, uint32_t max_q, const float* __restrict__ depth, const uint2* __restrict__ hpn, const uint32_t* __restrict__ rad, uint32_t* __restrict__ queries, uint32_t* __restrict__ count) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  uint32_t q = (uint32_t)y * (uint32_t)w + (uint32_t)x;
  if (q == 0) {
    uint32_t n = (uint32_t)w * (uint32_t)h;
    *count = n < max_q ? n : max_q;
  }
  if (q >= max_q) return;
  if (depth[q] == 0.0f) {
    store(queries, q, make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u));
    return;
  }
  uint2 e = hpn[q];
  f3 pos = hpn_pos(e.x, e.y);
  f3 nrm = hpn_normal(e.y);
  VertexKey k = vertex_key(pos, nrm, mk3(fp.view_pos[0], fp.view_pos[1], fp.view_pos[2]), bucket_mask, key_mode);
  store(queries, q, make_uint4(as_uint(pos.x), as_uint(pos.y), as_uint(pos.z), normal_encode_oct_u32(nrm)),
        make_uint4(k.hash, k.checksum, rad[q], 0u));
}
};

// ------------------------------------------------------------------ decay

// hash_grid_decay.hlsl:13-129, one thread per bucket (16 cells).
struct HgDecayF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t num_buckets, uint32_t* __restrict__ decay_words, uint4* __restrict__ storage) {
  uint32_t b = (uint32_t)x0 + threadIdx.x;
  if (b >= num_buckets) return;
  const uint32_t base = b * 16u;
  uint32_t mask = 0;
  uint32_t local[4] = {0u, 0u, 0u, 0u};
  uint32_t set = 0;
  while (set < 4u) {
    uint32_t set_addr = base + set * 4u;
    uint32_t packed = decay_words[set_addr >> 2];
    if (packed == 0u) break;
    uint32_t updated = 0;
    uint32_t dv = 0;
    for (uint32_t i = 0; i < 4u; ++i) {
      uint32_t sh = i * 8u;
      dv = (packed >> sh) & 0xFFu;
      if (dv == 0u) break;
      dv = dv - 1u;
      if (dv == 0u) {
        storage[set_addr + i] = make_uint4(0u, 0u, 0u, 0u);
      } else {
        updated |= dv << sh;
        mask |= 1u << (set * 4u + i);
      }
    }
    local[set] = updated;
    ++set;
    if (dv == 0u) break;
  }
  if (mask != 0u) {
    while (true) {
      uint32_t last = 31u - (uint32_t)__clz(mask);
      uint32_t first = (uint32_t)__ffs(~mask) - 1u;
      if (first < last) {
        uint32_t src = last >> 2, dst = first >> 2;
        uint32_t lsh = (last & 3u) * 8u;
        uint32_t dv = local[src] >> lsh;
        local[src] ^= dv << lsh;
        uint32_t fsh = (first & 3u) * 8u;
        local[dst] |= dv << fsh;
        storage[base + first] = storage[base + last];
        storage[base + last] = make_uint4(0u, 0u, 0u, 0u);
        mask |= 1u << first;
        mask ^= 1u << last;
      } else {
        break;
      }
    }
  }
  for (uint32_t i = 0; i < set; ++i) decay_words[(base >> 2) + i] = local[i];
}
};

// ------------------------------------------------------------------ select

struct SelectScratch {
  uint32_t* need_count;   // [num_buckets]
  uint32_t* need_offset;  // [num_buckets]
  uint32_t* total;        // [2]: miss-list length, number of buckets with misses
  uint32_t* list;         // [max_queries]
  uint32_t* buckets;      // [num_buckets]: the buckets with misses (any order)
  uint32_t* miss_bits;    // [max_queries / 32]: bit q of the queries that need an insertion
};

__host__ __device__ inline size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

static SelectScratch carve(const HashGridDims& d, void* base) {
  SelectScratch s;
  char* p = (char*)base;
  s.need_count = (uint32_t*)p;
  p += align256((size_t)d.num_buckets() * 4);
  s.need_offset = (uint32_t*)p;
  p += align256((size_t)d.num_buckets() * 4);
  s.total = (uint32_t*)p;
  p += 256;
  s.list = (uint32_t*)p;
  p += align256((size_t)d.max_queries * 4);
  s.buckets = (uint32_t*)p;
  p += align256((size_t)d.num_buckets() * 4);
  s.miss_bits = (uint32_t*)p;
  return s;
}

size_t hg_select_scratch_bytes(const HashGridDims& d) {
  return 3 * align256((size_t)d.num_buckets() * 4) + 256 + align256((size_t)d.max_queries * 4) +
         align256(((size_t)d.max_queries + 31) / 32 * 4);
}

__device__ __forceinline__ uint32_t select_word(uint32_t q, uint32_t frame_hash, uint32_t qbits) {
  uint32_t st = jenkins_hash(q ^ frame_hash);
  uint32_t r = lcg_xorshift(st);
  uint32_t score = r & (0xFFFFFFFFu << (qbits + 1u));
  return score | 0x80000000u | q;
}

// Probe of hash_grid_find_or_insert before any insertion: 0..15 = hit slot,
// 16 = needs an insertion (an empty slot exists), 17 = bucket full.
__device__ __forceinline__ uint32_t probe(const uint4* __restrict__ storage, uint32_t base, uint32_t c) {
  for (uint32_t k = 0; k < 16u; ++k) {
    uint32_t cs = storage[base + k].x;
    if (cs == c) return k;
    if (cs == 0u) return 16u;
  }
  return 17u;
}

// Probe: a query whose cell exists selects it at once (InterlockedMax); a query that
// needs an insertion counts itself in its bucket and sets its bit in miss_bits (one
// word per warp, every word of the launch written), so that the scatter pass visits
// only the misses.
struct HgSelProbeF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t max_q, const uint32_t* __restrict__ queries, const uint32_t* __restrict__ count, const uint4* __restrict__ storage, uint32_t* __restrict__ selection, uint32_t frame_hash, uint32_t qbits, uint32_t* __restrict__ need_count, uint32_t* __restrict__ miss_bits) {
  const uint32_t q = (uint32_t)x0 + threadIdx.x;
  uint32_t n = *count;
  n = n < max_q ? n : max_q;
  bool miss = false;
  if (q < n) {
    const uint4 rec1 = ((const uint4*)(queries + (size_t)q * Q_WORDS))[1];
    const uint32_t c = rec1.y;
    if (c != 0u) {
      const uint32_t base = rec1.x * 16u;
      const uint32_t k = probe(storage, base, c);
      if (k < 16u) {
        atomicMax(selection + base + k, select_word(q, frame_hash, qbits));
      } else if (k == 16u) {
        atomicAdd(need_count + rec1.x, 1u);
        miss = true;
      }
    }
  }
  const uint32_t bits = __ballot_sync(0xFFFFFFFFu, miss);
  if ((threadIdx.x & 31u) == 0u && q < max_q) miss_bits[q >> 5] = bits;
}
};

// Segment allocation: block-aggregated (one atomic per block and counter) offsets
// of the buckets' miss segments and the list of buckets with misses.
struct HgSelAllocF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t num_buckets, uint32_t* __restrict__ need_count, uint32_t* __restrict__ need_offset, uint32_t* __restrict__ total, uint32_t* __restrict__ buckets) {
  __shared__ uint32_t s_seg[kBlock1D / 32], s_act[kBlock1D / 32], s_base[2];
  const uint32_t b = (uint32_t)x0 + threadIdx.x;
  const uint32_t n = b < num_buckets ? need_count[b] : 0u;
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const uint32_t act = __ballot_sync(0xFFFFFFFFu, n != 0u);
  uint32_t incl = n;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  if (lane == 31u) {
    s_seg[wid] = incl;
    s_act[wid] = (uint32_t)__popc(act);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ts = 0u, ta = 0u;
    for (uint32_t w = 0; w < kBlock1D / 32; ++w) {
      const uint32_t vs = s_seg[w], va = s_act[w];
      s_seg[w] = ts;
      s_act[w] = ta;
      ts += vs;
      ta += va;
    }
    s_base[0] = ts ? atomicAdd(total, ts) : 0u;
    s_base[1] = ta ? atomicAdd(total + 1, ta) : 0u;
  }
  __syncthreads();
  if (n != 0u) {
    need_offset[b] = s_base[0] + s_seg[wid] + incl - n;
    need_count[b] = 0u;
    buckets[s_base[1] + s_act[wid] + (uint32_t)__popc(act & ((1u << lane) - 1u))] = b;
  }
  __syncthreads();  // the shared words are reused by the block's next tile (persistent launches)
}
};

// Scatter of the misses (the bits of miss_bits) into their buckets' segments.
struct HgSelScatterF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t max_q, const uint32_t* __restrict__ queries, const uint32_t* __restrict__ miss_bits, uint32_t* __restrict__ need_count, const uint32_t* __restrict__ need_offset, uint32_t* __restrict__ list) {
  const uint32_t q = (uint32_t)x0 + threadIdx.x;
  if (q >= max_q || !((miss_bits[q >> 5] >> (q & 31u)) & 1u)) return;
  const uint4 rec1 = ((const uint4*)(queries + (size_t)q * Q_WORDS))[1];
  uint32_t pos = atomicAdd(need_count + rec1.x, 1u);
  list[need_offset[rec1.x] + pos] = q;
}
};

struct HgSelResolveF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t n_warps, const uint32_t* __restrict__ queries, uint4* __restrict__ storage, uint32_t* __restrict__ selection, const uint32_t* __restrict__ need_count, const uint32_t* __restrict__ need_offset, uint32_t* __restrict__ list, uint32_t frame_hash, uint32_t qbits, const uint32_t* __restrict__ total, const uint32_t* __restrict__ buckets) {
  // n_warps warps loop over the buckets with misses (their order does not matter:
  // buckets are disjoint).
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t n_active = total[1];
  for (uint32_t wi = ((uint32_t)x0 + threadIdx.x) >> 5; wi < n_active; wi += n_warps) {
    resolve_bucket(buckets[wi], lane, queries, storage, selection, need_count, need_offset, list, frame_hash,
                   qbits);
  }
}
  static __device__ __forceinline__ void resolve_bucket(uint32_t bucket, uint32_t lane, const uint32_t* __restrict__ queries, uint4* __restrict__ storage, uint32_t* __restrict__ selection, const uint32_t* __restrict__ need_count, const uint32_t* __restrict__ need_offset, uint32_t* __restrict__ list, uint32_t frame_hash, uint32_t qbits) {
  uint32_t n = need_count[bucket];
  if (n == 0u) return;
  uint32_t off = need_offset[bucket];
  uint32_t base = bucket * 16u;
  uint32_t cs = lane < 16u ? storage[base + lane].x : 0xFFFFFFFFu;  // lanes >= 16 never match
  if (n <= 32u) {
    // At most one miss per lane: the rounds run on registers.
    const uint32_t q = lane < n ? list[off + lane] : 0xFFFFFFFFu;
    const uint32_t qc = lane < n ? queries[(size_t)q * Q_WORDS + Q_CHECK] : 0u;
    bool open = lane < n;
    while (true) {
      const uint32_t qmin = __reduce_min_sync(0xFFFFFFFFu, open ? q : 0xFFFFFFFFu);
      if (qmin == 0xFFFFFFFFu) break;
      const uint32_t owner = (uint32_t)__ffs(__ballot_sync(0xFFFFFFFFu, open && q == qmin)) - 1u;
      const uint32_t c = __shfl_sync(0xFFFFFFFFu, qc, owner);
      const uint32_t hit = __ballot_sync(0xFFFFFFFFu, lane < 16u && (cs == c || cs == 0u));
      if (hit == 0u) break;  // bucket full: every remaining query fails
      const uint32_t k = (uint32_t)__ffs(hit) - 1u;
      if (__shfl_sync(0xFFFFFFFFu, cs, k) == 0u && lane == k) {
        cs = c;
        storage[base + k].x = c;
      }
      const bool mine = open && qc == c;
      const uint32_t m = __reduce_max_sync(0xFFFFFFFFu, mine ? select_word(q, frame_hash, qbits) : 0u);
      if (lane == 0u) atomicMax(selection + base + k, m);
      open = open && !mine;
    }
    return;
  }
  const uint32_t RESOLVED = 0x80000000u;
  for (int round = 0; round < 17; ++round) {
    uint32_t qmin = 0xFFFFFFFFu;
    for (uint32_t j = lane; j < n; j += 32u) {
      uint32_t q = list[off + j];
      if (!(q & RESOLVED)) qmin = q < qmin ? q : qmin;
    }
    for (int o = 16; o > 0; o >>= 1) {
      uint32_t other = __shfl_xor_sync(0xFFFFFFFFu, qmin, o);
      qmin = other < qmin ? other : qmin;
    }
    if (qmin == 0xFFFFFFFFu) break;
    uint32_t c = queries[(size_t)qmin * Q_WORDS + Q_CHECK];
    uint32_t hit = __ballot_sync(0xFFFFFFFFu, lane < 16u && (cs == c || cs == 0u));
    if (hit == 0u) break;  // bucket full: every remaining query fails
    uint32_t k = (uint32_t)__ffs(hit) - 1u;
    uint32_t kcs = __shfl_sync(0xFFFFFFFFu, cs, k);
    if (kcs == 0u) {
      if (lane == k) {
        cs = c;
        storage[base + k].x = c;
      }
    }
    uint32_t m = 0u;
    for (uint32_t j = lane; j < n; j += 32u) {
      uint32_t q = list[off + j];
      if (q & RESOLVED) continue;
      if (queries[(size_t)q * Q_WORDS + Q_CHECK] != c) continue;
      const uint32_t sw = select_word(q, frame_hash, qbits);
      m = sw > m ? sw : m;
      list[off + j] = q | RESOLVED;
    }
    // One atomic per round: the maximum over the lanes' queries of this checksum.
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    if (lane == 0u) atomicMax(selection + base + k, m);
    __syncwarp();
  }
}
};

// ----------------------------------------------------------------- compact

// hash_grid_query_compact.hlsl:23-63 as the shader does it: block-local append in
// cell order, one global atomic per block (the blocks' order varies from run to run).
struct HgCompactF {
  static __device__ __forceinline__ void run(int x0, int y0, uint32_t num_cells, uint32_t qmask, const uint32_t* __restrict__ selection, uint32_t* __restrict__ idx, uint32_t* __restrict__ addr, uint32_t* __restrict__ count) {
  __shared__ uint32_t warp_cnt[kMaxThreads / 32];
  __shared__ uint32_t block_base;
  const int n_warps = (int)blockDim.x >> 5;
  uint32_t c = (uint32_t)x0 + threadIdx.x;
  uint32_t sel = c < num_cells ? selection[c] : 0u;
  uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint32_t bal = __ballot_sync(0xFFFFFFFFu, sel != 0u);
  if (lane == 0) warp_cnt[wid] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int k = 0; k < n_warps; ++k) {
      uint32_t v = warp_cnt[k];
      warp_cnt[k] = tot;
      tot += v;
    }
    block_base = tot ? atomicAdd(count, tot) : 0u;
  }
  __syncthreads();
  if (sel != 0u) {
    uint32_t pos = block_base + warp_cnt[wid] + __popc(bal & ((1u << lane) - 1u));
    idx[pos] = sel & qmask;
    addr[pos] = c;
  }
}
};

// hash_grid_query_compact.hlsl:23-63: the selected queries of all cells, listed in
// cell order (the shader appends per block through one atomic, so its order varies
// from run to run; the traced cache update derives each ray from the list position).
struct HgCompactSel {
  struct Args {
    const uint32_t* selection;
    uint32_t qmask;
    uint32_t* idx;
    uint32_t* addr;
  };
  static __device__ __forceinline__ bool flag(const Args& a, uint32_t c) { return a.selection[c] != 0u; }
  static __device__ __forceinline__ void emit(const Args& a, uint32_t c, uint32_t rank) {
    a.idx[rank] = a.selection[c] & a.qmask;
    a.addr[rank] = c;
  }
};

// ------------------------------------------------------------------ update

// hash_grid_raygen.hlsl:71-86 with the traced radiance supplied by the query.
struct HgUpdateF {
  static __device__ __forceinline__ void run(int x0, int y0, const uint32_t* __restrict__ queries, const uint32_t* __restrict__ idx, const uint32_t* __restrict__ addr, const uint32_t* __restrict__ count, uint4* __restrict__ storage, uint8_t* __restrict__ decay) {
  uint32_t k = (uint32_t)x0 + threadIdx.x;
  if (k >= *count) return;
  uint32_t q = idx[k], a = addr[k];
  f3 L = unpack_r11g11b10(queries[(size_t)q * Q_WORDS + Q_RAD]);
  uint4 cell = storage[a];
  f3 prev = mk3(as_float(cell.y), as_float(cell.z), as_float(cell.w));
  const float bf = 1.0f / 16.0f;
  f3 bl = L * bf + prev * (1.0f - bf);
  storage[a] = make_uint4(cell.x, as_uint(bl.x), as_uint(bl.y), as_uint(bl.z));
  decay[a] = 10;
}
};

// ------------------------------------------------------------------- find

struct HgFindF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, uint32_t bucket_mask, uint32_t key_mode, const uint4* __restrict__ storage, uint32_t n, const float* __restrict__ pos, const float* __restrict__ nrm, uint32_t* __restrict__ out_addr, float4* __restrict__ out_rad) {
  uint32_t i = (uint32_t)x0 + threadIdx.x;
  if (i >= n) return;
  f3 p = mk3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  f3 nn = mk3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
  VertexKey k = vertex_key(p, nn, mk3(fp.view_pos[0], fp.view_pos[1], fp.view_pos[2]), bucket_mask, key_mode);
  uint32_t base = k.hash * 16u;
  uint32_t found = 0xFFFFFFFFu;
  uint4 cell = make_uint4(0u, 0u, 0u, 0u);
  for (uint32_t s = 0; s < 16u; ++s) {
    uint4 c = storage[base + s];
    if (c.x == k.checksum) {
      found = base + s;
      cell = c;
      break;
    }
    if (c.x == 0u) break;
  }
  out_addr[i] = found;
  if (out_rad)
    out_rad[i] = make_float4(as_float(cell.y), as_float(cell.z), as_float(cell.w), found != 0xFFFFFFFFu ? 1.0f : 0.0f);
}
};

// ------------------------------------------------------------ visualize

// hash_grid_visualize.hlsl:16-65: the cache cell of each pixel's surface point (key
// from the position; key mode 1 also the G-buffer normal's octant), shown as its
// radiance or as a colour code from the checksum; no geometry: 0; no cell: (1, 0, 1)
// or, with the colour code, 0. Output R11G11B10.
struct HgVisualizeF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, uint32_t bucket_mask, uint32_t key_mode, const float* __restrict__ depth, const uint32_t* __restrict__ gbuf, const uint4* __restrict__ storage, uint32_t color_code, uint32_t* __restrict__ out) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  const float d = depth[i];
  if (d == 0.0f) {
    out[i] = 0u;
    return;
  }
  const f3 pos = depth_to_position(fp.inv_view_proj, x, y, w, h, d);
  const f3 nrm = gbuffer_normal(gbuf[(size_t)w * h + i]);
  const VertexKey k = vertex_key(pos, nrm, vpos3(fp.view_pos), bucket_mask, key_mode);
  const uint32_t base = k.hash * 16u;
  f3 color = color_code ? mk3(0.0f) : mk3(1.0f, 0.0f, 1.0f);
  for (uint32_t s = 0; s < 16u; ++s) {
    const uint4 c = storage[base + s];
    if (c.x == k.checksum) {
      if (color_code) {
        const uint32_t code = k.checksum;
        color = mk3(div_u8_255(code & 0xFFu), div_u8_255((code >> 8) & 0xFFu),
                    div_u8_255(((code >> 16) ^ (code >> 24)) & 0xFFu));
      } else {
        color = mk3(as_float(c.y), as_float(c.z), as_float(c.w));
      }
      break;
    }
    if (c.x == 0u) break;
  }
  out[i] = pack_r11g11b10(color);
}
};

// --------------------------------------------------------------- launchers

void launch_hg_visualize(const Exec& ex, const vlt_frame_params& fp, int w, int h, const HashGridDims& d,
                         uint32_t key_mode, const float* depth, const uint32_t* gbuf, const uint32_t* storage,
                         uint32_t color_code, uint32_t* out) {
  launch2d<HgVisualizeF>(ex, "hg_visualize", w, h, fp, w, h, d.num_buckets() - 1u, key_mode, depth, gbuf,
                         (const uint4*)storage, color_code, out);
}


void launch_hg_emit(const Exec& ex, const vlt_frame_params& fp, int w, int h, const HashGridDims& d,
                    uint32_t key_mode, const float* depth, const uint32_t* hpn, const uint32_t* rad,
                    uint32_t* queries, uint32_t* count) {
  if (((uintptr_t)queries & 31u) == 0)
    launch2d<HgEmitF<true>>(ex, "hg_emit", w, h, fp, w, h, d.num_buckets() - 1u, key_mode, d.max_queries, depth,
                            (const uint2*)hpn, rad, queries, count);
  else
    launch2d<HgEmitF<false>>(ex, "hg_emit", w, h, fp, w, h, d.num_buckets() - 1u, key_mode, d.max_queries, depth,
                             (const uint2*)hpn, rad, queries, count);
}

void launch_hg_decay(const Exec& ex, const HashGridDims& d, uint8_t* decay, uint32_t* storage) {
  uint32_t nb = d.num_buckets();
  launch1d<HgDecayF>(ex, "hg_decay", nb, nb, (uint32_t*)decay, (uint4*)storage);
}

void launch_hg_select(const Exec& ex, const HashGridDims& d, const uint32_t* queries, const uint32_t* count,
                      uint32_t* storage, uint32_t* selection, uint32_t frame_hash, void* scratch) {
  SelectScratch sc = carve(d, scratch);
  uint32_t nb = d.num_buckets();
  uint32_t qb = d.query_bits();
  ex_fill32(ex, sc.need_count, 0u, (size_t)nb * 4);
  ex_fill32(ex, sc.total, 0u, 8);
  uint32_t nq = d.max_queries;
  launch1d<HgSelProbeF>(ex, "hg_select", nq, nq, queries, count, (const uint4*)storage, selection, frame_hash, qb,
                        sc.need_count, sc.miss_bits);
  launch1d<HgSelAllocF>(ex, "hg_select", nb, nb, sc.need_count, sc.need_offset, sc.total, sc.buckets);
  launch1d<HgSelScatterF>(ex, "hg_select", nq, nq, queries, (const uint32_t*)sc.miss_bits, sc.need_count,
                          (const uint32_t*)sc.need_offset, sc.list);
  // One warp per bucket with misses, at most a full device of warps looping over them.
  const uint64_t cap = (uint64_t)device_sm_count() * 64u;
  const uint32_t n_warps = (uint32_t)(nb < cap ? nb : cap);
  launch1d<HgSelResolveF>(ex, "hg_select", n_warps * 32u, n_warps, queries, (uint4*)storage, selection,
                          (const uint32_t*)sc.need_count, (const uint32_t*)sc.need_offset, sc.list, frame_hash, qb,
                          (const uint32_t*)sc.total, (const uint32_t*)sc.buckets);
}

void launch_hg_compact(const Exec& ex, const HashGridDims& d, const uint32_t* selection, uint32_t* idx,
                       uint32_t* addr, uint32_t* count, uint32_t* scratch) {
  if (!scratch) {
    uint32_t nc = d.num_cells();
    uint32_t qmask = (1u << d.query_bits()) - 1u;
    launch1d<HgCompactF>(ex, "hg_compact", nc, nc, qmask, selection, idx, addr, count);
    return;
  }
  HgCompactSel::Args a = {selection, (1u << d.query_bits()) - 1u, idx, addr};
  launch_compact<HgCompactSel>(ex, "hg_compact", d.num_cells(), a, scratch, count);
}

void launch_hg_update(const Exec& ex, const HashGridDims& d, const uint32_t* queries, const uint32_t* idx,
                      const uint32_t* addr, const uint32_t* count, uint32_t* storage, uint8_t* decay) {
  uint32_t nmax = d.max_queries < d.num_cells() ? d.max_queries : d.num_cells();
  launch1d<HgUpdateF>(ex, "hg_update", nmax, queries, idx, addr, count, (uint4*)storage, decay);
}

void launch_hg_find(const Exec& ex, const vlt_frame_params& fp, const HashGridDims& d, uint32_t key_mode,
                    const uint32_t* storage, uint32_t n, const float* pos, const float* nrm, uint32_t* out_addr,
                    float* out_rad) {
  launch1d<HgFindF>(ex, "hg_find", n, fp, d.num_buckets() - 1u, key_mode, (const uint4*)storage, n, pos, nrm,
                    out_addr, (float4*)out_rad);
}

// ------------------------------------------- query select without allocation

// Scratch for vlt_hg_query_select_noalloc: a fixed array in the library's own
// device memory, so that callers who cannot allocate device memory can still run
// the query selection. It exists once per GPU that loads the library and stays
// until the process exits. Every call uses the same array.
static __device__ __align__(256) unsigned char g_hg_select_scratch[VLT_HG_SELECT_NOALLOC_SCRATCH_BYTES];

// Device address of g_hg_select_scratch, looked up once per device (host code
// cannot use the symbol itself as a device pointer). The address is kept for the
// life of the process; after a cudaDeviceReset the module is loaded again and the
// kept address is stale, so the entry point is documented as unusable after one.
static void* g_hg_select_scratch_ptr[64];
static bool g_hg_select_scratch_ready[64];
static std::mutex g_hg_select_scratch_mutex;

}  // namespace vlt

extern "C" vlt_status vlt_hg_query_select_noalloc(uint32_t log2_buckets, uint32_t max_queries,
                                                  const uint32_t* queries, const uint32_t* query_count,
                                                  uint32_t* rw_storage, uint32_t* rw_selection, uint32_t frame_hash,
                                                  void* stream) {
  using namespace vlt;
  if (log2_buckets < 4 || log2_buckets > 24 || max_queries == 0 || max_queries > (1u << 30) || !queries ||
      !query_count || !rw_storage || !rw_selection) {
    set_last_error("vlt_hg_query_select_noalloc: log2_buckets must be in [4, 24], max_queries in [1, 2^30], and "
                   "every buffer pointer non-null");
    return VLT_ERR_INVALID_ARG;
  }
  HashGridDims d = {log2_buckets, max_queries};
  if (hg_select_scratch_bytes(d) > (size_t)VLT_HG_SELECT_NOALLOC_SCRATCH_BYTES) {
    set_last_error("vlt_hg_query_select_noalloc: 2^log2_buckets buckets and max_queries need more scratch than the "
                   "fixed VLT_HG_SELECT_NOALLOC_SCRATCH_BYTES; use vlt_hg_query_select with caller scratch");
    return VLT_ERR_INVALID_ARG;
  }
  int dev = 0;
  vlt_status st = cuda_status(cudaGetDevice(&dev));
  if (st != VLT_OK) return st;
  if (dev < 0 || dev >= 64) {
    set_last_error("vlt_hg_query_select_noalloc: device ordinals of 64 and above are not supported");
    return VLT_ERR_INVALID_ARG;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_hg_select_scratch_mutex);
    if (!g_hg_select_scratch_ready[dev]) {
      // First call on this device: resolve the array's device address (device `dev`
      // is current here).
      void* p = nullptr;
      st = cuda_status(cudaGetSymbolAddress(&p, g_hg_select_scratch));
      if (st != VLT_OK) return st;
      g_hg_select_scratch_ptr[dev] = p;
      g_hg_select_scratch_ready[dev] = true;
    }
    scratch = g_hg_select_scratch_ptr[dev];
  }
  // launch_hg_select clears the per-bucket counters it needs at zero before use;
  // the rest of the scratch is fully rewritten before it is read.
  Exec ex;
  ex.stream = (cudaStream_t)stream;
  launch_hg_select(ex, d, queries, query_count, rw_storage, rw_selection, frame_hash, scratch);
  return cuda_status(cudaGetLastError());
}
