// Stand-in for slate::Tile (include/slate/Tile.hh) with the members SLATE's
// tile panel code uses: a column-major view (data, mb x nb, stride) with
// element access.  Test infrastructure only.
#ifndef ORACLE_REFSHIM_SLATE_TILE_HH
#define ORACLE_REFSHIM_SLATE_TILE_HH
#include <cstdint>
#include "slate/types.hh"
namespace slate {
template <typename T> class Tile {
public:
    Tile() = default;
    Tile(int64_t mb, int64_t nb, T* data, int64_t stride) : mb_(mb), nb_(nb), stride_(stride), data_(data) {}
    int64_t mb() const { return mb_; }
    int64_t nb() const { return nb_; }
    int64_t stride() const { return stride_; }
    int64_t rowIncrement() const { return stride_; }
    int64_t colIncrement() const { return 1; }
    T* data() const { return data_; }
    T operator()(int64_t i, int64_t j) const { return data_[i + j * stride_]; }
    T& at(int64_t i, int64_t j) const { return data_[i + j * stride_]; }
private:
    int64_t mb_ = 0, nb_ = 0, stride_ = 1;
    T* data_ = nullptr;
};
} // namespace slate
#endif
