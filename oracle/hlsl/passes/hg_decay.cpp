// ORACLE — test infrastructure only: restir/hash_grid_decay.hlsl compiled from the
// reference's text, behind the oracle's vlto_hg_decay signature (decay bytes, 16-byte
// cells {checksum, radiance}). The shader's grid has 2^16 buckets of 16 cells.
#include "harness.hpp"

namespace hlsl {
namespace ref_hg_decay {
#include "shader/restir/hash_grid_decay.hlsl"
}
}  // namespace hlsl

extern "C" int vltr_hg_decay(uint32_t log2_buckets, uint8_t* decay, uint32_t* storage) {
  namespace S = hlsl::ref_hg_decay;
  static_assert(sizeof(S::HashGridCell) == 16, "HashGridCell is 16 bytes");
  if (log2_buckets != 16) return -1;  // HASH_GRID_NUM_BUCKETS is 65536 in the shader
  S::rw_decay_buffer.data = decay;
  S::rw_decay_buffer.bytes = HASH_GRID_NUM_CELLS;
  S::rw_storage_buffer.data = (S::HashGridCell*)storage;
  S::rw_storage_buffer.count = HASH_GRID_NUM_CELLS;
  // One thread per bucket (hash_grid_decay.hlsl:13); buckets are disjoint.
  hlsl::dispatch(S::hlsl_entry, hlsl::uint3(S::hlsl_numthreads[0], 1u, 1u),
                 hlsl::uint3(HASH_GRID_NUM_BUCKETS / S::hlsl_numthreads[0], 1u, 1u), false, false);
  return 0;
}
