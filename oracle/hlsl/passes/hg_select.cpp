// ORACLE — test infrastructure only: restir/hash_grid_query_select.hlsl compiled from
// the reference's text, behind the oracle's vlto_hg_query_select signature (8-word
// query records whose first six words are HashGridQuery). Threads run one at a time in
// query order, the order that defines the insertion result.
#include <vector>

#include "harness.hpp"

namespace hlsl {
namespace ref_hg_select {
#include "shader/restir/hash_grid_query_select.hlsl"
}
}  // namespace hlsl

extern "C" int vltr_hg_query_select(uint32_t log2_buckets, uint32_t max_q, const uint32_t* queries,
                                    const uint32_t* count, uint32_t* storage, uint32_t* selection,
                                    uint32_t frame_hash) {
  namespace S = hlsl::ref_hg_select;
  static_assert(sizeof(S::HashGridQuery) == 24, "HashGridQuery is 24 bytes");
  if (log2_buckets != 16 || max_q > HASH_GRID_MAX_NUM_QUERIES) return -1;
  std::vector<S::HashGridQuery> q(max_q);
  for (uint32_t i = 0; i < max_q; ++i) memcpy(&q[i], queries + 8 * (size_t)i, sizeof(S::HashGridQuery));
  S::hash_grid_query_buffer.data = q.data();
  S::hash_grid_query_buffer.count = max_q;
  S::hash_grid_query_counter_buffer.data = count;
  S::hash_grid_query_counter_buffer.count = 1;
  S::rw_hash_grid_storage_buffer.data = (S::HashGridCell*)storage;
  S::rw_hash_grid_storage_buffer.count = HASH_GRID_NUM_CELLS;
  S::rw_hash_grid_query_selection_buffer.data = selection;
  S::rw_hash_grid_query_selection_buffer.count = HASH_GRID_NUM_CELLS;
  S::pc.frame_hash = frame_hash;
  harness::run_1d_sequential(S::hlsl_entry, S::hlsl_numthreads, max_q);
  return 0;
}
