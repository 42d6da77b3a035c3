// Stand-in for the src/internal/internal.hh names SLATE's tile panel code
// uses: internal::AuxPivot (pivot record: tile index, offset, local tile
// index, value, owner rank).  Test infrastructure only.
#ifndef ORACLE_REFSHIM_INTERNAL_HH
#define ORACLE_REFSHIM_INTERNAL_HH
#include <cstdint>
#include "slate/types.hh"
namespace slate {
namespace internal {
template <typename T> class AuxPivot {
public:
    AuxPivot() = default;
    AuxPivot(int64_t tile_index, int64_t element_offset, int64_t local_tile_index, T value, int rank)
        : tile_index_(tile_index), element_offset_(element_offset), local_tile_index_(local_tile_index),
          value_(value), rank_(rank) {}
    int64_t tileIndex() { return tile_index_; }
    int64_t elementOffset() { return element_offset_; }
    int64_t localTileIndex() { return local_tile_index_; }
    T value() { return value_; }
    int rank() { return rank_; }
private:
    int64_t tile_index_ = 0, element_offset_ = 0, local_tile_index_ = 0;
    T value_{};
    int rank_ = 0;
};
} // namespace internal
} // namespace slate
#endif
