// slate_gb300.hh -- SLATE's C++ driver API for the single-GPU solve path,
// header-only over the C ABI of libslate_gb300.so.
//
// Names, argument order and meaning follow include/slate/slate.hh:503-770
// (gesv, getrf, getrs, gesv_mixed, gesv_mixed_gmres, gesv_rbt, posv, potrf,
// potrs, posv_mixed, posv_mixed_gmres, gecondest, pocondest) and the
// simplified API include/slate/simplified_api.hh (lu_solve, lu_factor,
// lu_solve_using_factor, chol_solve, chol_factor, chol_solve_using_factor),
// with SLATE's Option keys (include/slate/enums.hh:453-490), Pivot
// (include/slate/types.hh:84-117) and its tile storage model: a matrix is a
// shallow handle on a shared map from tile (i, j) and device to Tile
// instances, each with its MOSI state (include/slate/BaseMatrix.hh:360-430,
// 2791-2830; include/slate/internal/MatrixStorage.hh:35-470).
//
// A C++ caller of SLATE on a 1 x 1 grid with Target::Devices changes
// `slate::` to `slate_gb300::`.  Matrices may be
//  * fromLAPACK(m, n, A, lda, nb[, p, q]) on host or device memory,
//  * fromDevices(m, n, Aarray, 1, lda, nb[, p, q]),
//  * Matrix(m, n, nb, p, q) filled with insertLocalTiles(Target) or
//    tileInsert(i, j, device[, data, ld]) tile by tile,
// and the drivers run on the GPU whatever the origin: the tiles are gathered
// into one column-major device array (the caller's own array is used as it
// is when the matrix is one current device array), the driver runs there,
// and the results go back to each tile's home instance, which becomes the
// only valid one (MOSI Modified, every other instance Invalid), as after
// SLATE's tileUpdateAllOrigin.
//
// Differences: the grid must be 1 x 1 and mb = nb; device is 0 or HostNum;
// errors throw slate_gb300::Exception carrying the library's status (SLATE
// throws slate::Exception); the mixed solvers are double (and complex<double>
// for gesv_mixed, SLATE's own instantiations).
#pragma once

#include <complex>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "slate_gb300.h"

namespace slate_gb300 {

class Exception : public std::runtime_error {
public:
    explicit Exception(int status)
        : std::runtime_error(std::string("slate_gb300: ") + slt_status_string(status)), status_(status) {}
    int status() const { return status_; }
private:
    int status_;
};

inline void check(int status) { if (status != 0) throw Exception(status); }

enum class Option {
    Lookahead, BlockSize, InnerBlocking, MaxPanelThreads, Tolerance, Target, MaxIterations,
    UseFallbackSolver, PivotThreshold, MethodLU, Depth,
    FactorPrecision, Refine, Equilibrate          // this library's additions
};
enum class Target : char { Host = 'H', HostTask = 'T', HostNest = 'N', HostBatch = 'B', Devices = 'D' };
enum class MethodLU : char { Auto = '*', PartialPiv = 'P', CALU = 'C', NoPiv = 'N' };
enum class Uplo : char { Lower = 'L', Upper = 'U' };
enum class Norm : char { One = '1', Inf = 'I' };
// Tile coherency states of SLATE's MOSI protocol (include/slate/enums.hh).
enum class MOSI : char { Modified = 'M', OnHold = 'O', Shared = 'S', Invalid = 'I' };
enum class TileKind : char { Workspace = 'w', SlateOwned = 'o', UserOwned = 'u' };
enum class LayoutConvert : char { None = 'N', ColMajor = 'C', RowMajor = 'R' };
constexpr int HostNum = -1;

// The value of one option: SLATE's OptionValue holds an int64 or a double.
class OptionValue {
public:
    OptionValue(int64_t i) : i_(i), d_(double(i)) {}
    OptionValue(int i) : i_(i), d_(double(i)) {}
    OptionValue(double d) : i_(int64_t(d)), d_(d) {}
    OptionValue(bool b) : i_(b ? 1 : 0), d_(b ? 1.0 : 0.0) {}
    OptionValue(Target t) : i_(int64_t(t)), d_(double(int64_t(t))) {}
    OptionValue(MethodLU m) : i_(int64_t(m)), d_(double(int64_t(m))) {}
    int64_t i() const { return i_; }
    double d() const { return d_; }
private:
    int64_t i_;
    double d_;
};
using Options = std::map<Option, OptionValue>;

// Pivot of row k*nb + j: tile index relative to panel k and offset in that tile.
struct Pivot {
    int64_t tile_index = 0, element_offset = 0;
    Pivot() = default;
    Pivot(int64_t t, int64_t o) : tile_index(t), element_offset(o) {}
    int64_t tileIndex() const { return tile_index; }
    int64_t elementOffset() const { return element_offset; }
};
using Pivots = std::vector<std::vector<Pivot>>;

// ---------------------------------------------------------------------------
// Tiles and their storage.
template <typename T>
class Tile {
public:
    Tile() = default;
    Tile(int64_t mb, int64_t nb, T* data, int64_t stride, int device, TileKind kind)
        : mb_(mb), nb_(nb), stride_(stride), data_(data), device_(device), kind_(kind) {}
    int64_t mb() const { return mb_; }
    int64_t nb() const { return nb_; }
    int64_t stride() const { return stride_; }
    T* data() const { return data_; }
    int device() const { return device_; }
    TileKind kind() const { return kind_; }
    bool origin() const { return kind_ == TileKind::UserOwned; }
    // element access of a host tile (column-major)
    T operator()(int64_t i, int64_t j) const { return data_[i + j * stride_]; }
    T& at(int64_t i, int64_t j) const { return data_[i + j * stride_]; }
private:
    int64_t mb_ = 0, nb_ = 0, stride_ = 1;
    T* data_ = nullptr;
    int device_ = HostNum;
    TileKind kind_ = TileKind::Workspace;
};

namespace detail {

inline void copy_tile(void* dst, int64_t ldd, const void* src, int64_t lds, int64_t mb, int64_t nb, size_t esize)
{
    check(slt_memcpy2d(dst, size_t(ldd) * esize, src, size_t(lds) * esize, size_t(mb) * esize, size_t(nb)));
}

template <typename T> struct TypeCode;
template <> struct TypeCode<float> { static constexpr int value = 0; };
template <> struct TypeCode<double> { static constexpr int value = 1; };
template <> struct TypeCode<std::complex<float>> { static constexpr int value = 2; };
template <> struct TypeCode<std::complex<double>> { static constexpr int value = 3; };

}  // namespace detail

// The shared tile map of one matrix: tile (i, j) -> its instances by device
// (HostNum or 0), each with a MOSI state, and the tile's home (its origin, or
// where it was inserted).  SLATE-owned and workspace instances are freed with
// the storage.
template <typename T>
class MatrixStorage {
public:
    struct Instance {
        Tile<T> tile;
        MOSI state = MOSI::Invalid;
    };
    struct Node {
        std::map<int, Instance> inst;
        int home = HostNum;
    };
    MatrixStorage(int64_t m, int64_t n, int64_t nb) : m(m), n(n), nb(nb) {
        if (m < 0 || n < 0 || nb <= 0) throw Exception(SLT_ERR_ARG);
    }
    ~MatrixStorage() {
        for (auto& kv : tiles)
            for (auto& in : kv.second.inst) release(in.second.tile);
    }
    MatrixStorage(const MatrixStorage&) = delete;
    MatrixStorage& operator=(const MatrixStorage&) = delete;

    int64_t tileMb(int64_t i) const { return (i + 1) * nb <= m ? nb : m - i * nb; }
    int64_t tileNb(int64_t j) const { return (j + 1) * nb <= n ? nb : n - j * nb; }

    Tile<T> allocate(int64_t i, int64_t j, int device, TileKind kind) {
        const int64_t mb = tileMb(i), tnb = tileNb(j);
        T* p = nullptr;
        if (device == HostNum) {
            p = new T[size_t(mb > 0 ? mb : 1) * size_t(tnb > 0 ? tnb : 1)]();
        }
        else {
            void* v = nullptr;
            check(slt_device_malloc(sizeof(T) * size_t(mb > 0 ? mb : 1) * size_t(tnb > 0 ? tnb : 1), &v));
            p = static_cast<T*>(v);
        }
        return Tile<T>(mb, tnb, p, mb > 0 ? mb : 1, device, kind);
    }
    static void release(const Tile<T>& t) {
        if (t.kind() == TileKind::UserOwned || !t.data()) return;
        if (t.device() == HostNum) delete[] t.data();
        else slt_device_free(t.data());
    }

    int64_t m, n, nb;
    std::map<std::pair<int64_t, int64_t>, Node> tiles;
    // a matrix made from one column-major array (fromLAPACK / fromDevices)
    T* origin = nullptr;
    int64_t origin_ld = 0;
    int origin_device = HostNum;
};

// Operations common to Matrix and HermitianMatrix (slate::BaseMatrix).
template <typename T>
class BaseMatrix {
public:
    BaseMatrix() = default;
    int64_t m() const { return st_ ? st_->m : 0; }
    int64_t n() const { return st_ ? st_->n : 0; }
    int64_t mt() const { return st_ ? (st_->m + st_->nb - 1) / st_->nb : 0; }
    int64_t nt() const { return st_ ? (st_->n + st_->nb - 1) / st_->nb : 0; }
    int64_t tileMb(int64_t i) const { return st_->tileMb(i); }
    int64_t tileNb(int64_t j) const { return st_->tileNb(j); }
    bool tileIsLocal(int64_t, int64_t) const { return true; }     // 1 x 1 grid
    int tileRank(int64_t, int64_t) const { return 0; }
    int tileDevice(int64_t, int64_t) const { return 0; }
    int mpiRank() const { return 0; }
    int num_devices() const { return 1; }
    std::shared_ptr<MatrixStorage<T>> storage() const { return st_; }

    bool tileExists(int64_t i, int64_t j, int device = HostNum) const {
        auto it = st_->tiles.find({i, j});
        return it != st_->tiles.end() && it->second.inst.count(device);
    }
    // The tile's instance on `device` (SLATE's A(i, j, device)).
    Tile<T> operator()(int64_t i, int64_t j, int device = HostNum) const { return at(i, j, device); }
    Tile<T> at(int64_t i, int64_t j, int device = HostNum) const {
        auto& node = st_->tiles.at({i, j});
        auto it = node.inst.find(device);
        if (it == node.inst.end()) throw Exception(SLT_ERR_ARG);
        return it->second.tile;
    }
    MOSI tileState(int64_t i, int64_t j, int device = HostNum) const {
        auto& node = st_->tiles.at({i, j});
        auto it = node.inst.find(device);
        return it == node.inst.end() ? MOSI::Invalid : it->second.state;
    }
    // A SLATE-owned tile on `device` (SLATE's tileInsert(i, j, device)).
    Tile<T> tileInsert(int64_t i, int64_t j, int device = HostNum) {
        check_index(i, j, device);
        auto& node = st_->tiles[{i, j}];
        if (node.inst.count(device)) throw Exception(SLT_ERR_ARG);
        Tile<T> t = st_->allocate(i, j, device, TileKind::SlateOwned);
        const bool first = node.inst.empty();
        node.inst[device] = {t, first ? MOSI::Modified : MOSI::Invalid};
        if (first) node.home = device;
        return t;
    }
    // A user-owned tile at data with leading dimension ld (SLATE's
    // tileInsert(i, j, device, data, ld)); it becomes the tile's home.
    Tile<T> tileInsert(int64_t i, int64_t j, int device, T* data, int64_t ld) {
        check_index(i, j, device);
        if (!data || ld < tileMb(i)) throw Exception(SLT_ERR_ARG);
        auto& node = st_->tiles[{i, j}];
        if (node.inst.count(device)) throw Exception(SLT_ERR_ARG);
        Tile<T> t(tileMb(i), tileNb(j), data, ld, device, TileKind::UserOwned);
        for (auto& in : node.inst) in.second.state = MOSI::Invalid;
        node.inst[device] = {t, MOSI::Modified};
        node.home = device;
        return t;
    }
    // Every tile, SLATE-owned, on the host (Target::Host*) or device 0
    // (Target::Devices) (SLATE's insertLocalTiles).
    void insertLocalTiles(Target origin = Target::Host) {
        const int dev = origin == Target::Devices ? 0 : HostNum;
        for (int64_t j = 0; j < nt(); ++j)
            for (int64_t i = 0; i < mt(); ++i)
                if (!tileExists(i, j, dev)) tileInsert(i, j, dev);
    }
    // MOSI: bring a valid copy of the tile to `device`.
    void tileGetForReading(int64_t i, int64_t j, int device = HostNum, LayoutConvert = LayoutConvert::None) {
        auto& node = st_->tiles.at({i, j});
        auto it = node.inst.find(device);
        if (it != node.inst.end() && it->second.state != MOSI::Invalid) return;
        typename MatrixStorage<T>::Instance* src = nullptr;
        for (auto& in : node.inst)
            if (in.second.state == MOSI::Modified || in.second.state == MOSI::Shared) { src = &in.second; break; }
        if (!src) throw Exception(SLT_ERR_ARG);             // no valid copy anywhere
        if (it == node.inst.end())
            it = node.inst.emplace(device, typename MatrixStorage<T>::Instance{
                     st_->allocate(i, j, device, TileKind::Workspace), MOSI::Invalid}).first;
        const Tile<T>& s = src->tile;
        const Tile<T>& d = it->second.tile;
        detail::copy_tile(d.data(), d.stride(), s.data(), s.stride(), s.mb(), s.nb(), sizeof(T));
        if (src->state == MOSI::Modified) src->state = MOSI::Shared;
        it->second.state = MOSI::Shared;
    }
    // MOSI: a valid copy on `device` that every other instance loses.
    void tileGetForWriting(int64_t i, int64_t j, int device = HostNum, LayoutConvert lc = LayoutConvert::None) {
        tileGetForReading(i, j, device, lc);
        tileModified(i, j, device);
    }
    void tileModified(int64_t i, int64_t j, int device = HostNum, bool = false) {
        auto& node = st_->tiles.at({i, j});
        if (!node.inst.count(device)) throw Exception(SLT_ERR_ARG);
        for (auto& in : node.inst) in.second.state = in.first == device ? MOSI::Modified : MOSI::Invalid;
    }
    void tileGetAllForReading(int device = HostNum, LayoutConvert lc = LayoutConvert::None) {
        for (auto& kv : st_->tiles) tileGetForReading(kv.first.first, kv.first.second, device, lc);
    }
    void tileGetAllForWriting(int device = HostNum, LayoutConvert lc = LayoutConvert::None) {
        for (auto& kv : st_->tiles) tileGetForWriting(kv.first.first, kv.first.second, device, lc);
    }
    // Copy the valid data back to the tile's home instance (the user's array).
    void tileUpdateOrigin(int64_t i, int64_t j) { tileGetForReading(i, j, st_->tiles.at({i, j}).home); }
    void tileUpdateAllOrigin() {
        for (auto& kv : st_->tiles) tileUpdateOrigin(kv.first.first, kv.first.second);
    }
    // Free the workspace instances (a valid home instance is kept up to date first).
    void releaseWorkspace() {
        tileUpdateAllOrigin();
        for (auto& kv : st_->tiles) {
            auto& node = kv.second;
            for (auto it = node.inst.begin(); it != node.inst.end();) {
                if (it->second.tile.kind() == TileKind::Workspace) {
                    MatrixStorage<T>::release(it->second.tile);
                    it = node.inst.erase(it);
                }
                else {
                    ++it;
                }
            }
        }
    }
    // legacy accessors: the origin array of fromLAPACK / fromDevices matrices
    T* data() const { return st_ ? st_->origin : nullptr; }
    int64_t stride() const { return st_ ? st_->origin_ld : 1; }

protected:
    void check_index(int64_t i, int64_t j, int device) const {
        if (!st_ || i < 0 || j < 0 || i >= mt() || j >= nt() || (device != HostNum && device != 0))
            throw Exception(SLT_ERR_ARG);
    }
    // one column-major array: every tile a user-owned view of it
    void attach_origin(T* A, int64_t lda) {
        const int dev = slt_is_device_pointer(A) ? 0 : HostNum;
        st_->origin = A;
        st_->origin_ld = lda;
        st_->origin_device = dev;
        for (int64_t j = 0; j < nt(); ++j)
            for (int64_t i = 0; i < mt(); ++i)
                tileInsert(i, j, dev, A + i * st_->nb + j * st_->nb * lda, lda);
    }
    std::shared_ptr<MatrixStorage<T>> st_;
};

template <typename T>
class Matrix : public BaseMatrix<T> {
public:
    Matrix() = default;
    // An empty m x n matrix of nb x nb tiles (tiles to be inserted).
    Matrix(int64_t m, int64_t n, int64_t nb, int p = 1, int q = 1, int64_t /*mpi_comm*/ = 0) {
        if (p != 1 || q != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        this->st_ = std::make_shared<MatrixStorage<T>>(m, n, nb);
    }
    static Matrix fromDevices(int64_t m, int64_t n, T** Aarray, int num_devices, int64_t lda, int64_t nb,
                              int p = 1, int q = 1) {
        if (num_devices != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return fromLAPACK(m, n, Aarray[0], lda, nb, p, q);
    }
    // The caller's column-major array, in host or device memory.
    static Matrix fromLAPACK(int64_t m, int64_t n, T* A, int64_t lda, int64_t nb, int p = 1, int q = 1) {
        if (lda < (m > 1 ? m : 1)) throw Exception(SLT_ERR_ARG);
        Matrix M(m, n, nb, p, q);
        M.attach_origin(A, lda);
        return M;
    }
    // Same shape and tile size, no tiles (SLATE's emptyLike).
    Matrix emptyLike() const { return Matrix(this->m(), this->n(), this->st_->nb); }
};

template <typename T>
class HermitianMatrix : public Matrix<T> {
public:
    HermitianMatrix() = default;
    HermitianMatrix(Uplo uplo, int64_t n, int64_t nb, int p = 1, int q = 1, int64_t mpi_comm = 0)
        : Matrix<T>(n, n, nb, p, q, mpi_comm), uplo_(uplo) {}
    static HermitianMatrix fromDevices(Uplo uplo, int64_t n, T** Aarray, int num_devices, int64_t lda,
                                       int64_t nb, int p = 1, int q = 1) {
        if (num_devices != 1) throw Exception(SLT_ERR_NOT_SUPPORTED);
        return fromLAPACK(uplo, n, Aarray[0], lda, nb, p, q);
    }
    static HermitianMatrix fromLAPACK(Uplo uplo, int64_t n, T* A, int64_t lda, int64_t nb, int p = 1, int q = 1) {
        if (lda < (n > 1 ? n : 1)) throw Exception(SLT_ERR_ARG);
        HermitianMatrix H(uplo, n, nb, p, q);
        H.attach_origin(A, lda);
        return H;
    }
    HermitianMatrix emptyLike() const { return HermitianMatrix(uplo_, this->n(), this->st_->nb); }
    Uplo uplo() const { return uplo_; }
private:
    Uplo uplo_ = Uplo::Lower;
};

namespace detail {

inline slt_options to_c(const Options& opts, int64_t nb)
{
    slt_options o;
    slt_options_default(&o);
    o.nb = nb;
    for (const auto& kv : opts) {
        switch (kv.first) {
            case Option::BlockSize:         break;              // the matrix's tile size rules, as in SLATE
            case Option::InnerBlocking:     o.ib = kv.second.i(); break;
            case Option::Lookahead:         o.lookahead = kv.second.i(); break;
            case Option::MaxIterations:     o.max_iterations = kv.second.i(); break;
            case Option::Tolerance:         o.tolerance = kv.second.d(); break;
            case Option::UseFallbackSolver: o.use_fallback = int(kv.second.i() != 0); break;
            case Option::PivotThreshold:    o.pivot_threshold = kv.second.d(); break;
            case Option::Depth:             o.depth = kv.second.i(); break;
            case Option::MethodLU:
                if (kv.second.i() == int64_t(MethodLU::NoPiv)) o.method_lu = 'N';
                if (kv.second.i() == int64_t(MethodLU::CALU)) o.method_lu = 'C';
                break;
            case Option::FactorPrecision:   o.factor_precision = int(kv.second.i()); break;
            case Option::Refine:            o.refine = int(kv.second.i()); break;
            case Option::Equilibrate:       o.equilibrate = int(kv.second.i()); break;
            default:                        break;              // Target, MaxPanelThreads: accepted
        }
    }
    return o;
}

// The matrix as one column-major device array for a driver call.  The
// caller's array itself when the matrix is one device array whose tiles are
// all current there; else a device workspace the tiles are gathered into.
// close() brings the driver's results back: into each tile's home instance,
// which becomes the only valid one.  With a triangle (Hermitian input) only
// that triangle of the results is written; the rest of each tile keeps its
// values.
template <typename T>
class DeviceArray {
public:
    DeviceArray(BaseMatrix<T>& A) : A_(A), st_(storage_of(A)) {
        if (st_.origin && st_.origin_device == 0 && all_home_current()) {
            p_ = st_.origin;
            ld_ = st_.origin_ld;
            return;
        }
        ld_ = st_.m > 1 ? st_.m : 1;
        void* v = nullptr;
        check(slt_device_malloc(sizeof(T) * size_t(ld_) * size_t(st_.n > 0 ? st_.n : 1), &v));
        p_ = static_cast<T*>(v);
        owned_ = true;
        for (int64_t j = 0; j < A.nt(); ++j)
            for (int64_t i = 0; i < A.mt(); ++i) {
                const Tile<T> t = valid_instance(i, j);
                copy_tile(p_ + i * st_.nb + j * st_.nb * ld_, ld_, t.data(), t.stride(), t.mb(), t.nb(), sizeof(T));
            }
    }
    ~DeviceArray() { if (owned_) slt_device_free(p_); }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    T* data() const { return p_; }
    int64_t ld() const { return ld_; }
    // tri: 0 all, 'L' lower triangle only, 'U' upper triangle only
    void close(char tri = 0) {
        if (owned_ && tri) {
            // keep the unreferenced triangle: refill it from the tiles' current values
            void* v = nullptr;
            check(slt_device_malloc(sizeof(T) * size_t(ld_) * size_t(st_.n > 0 ? st_.n : 1), &v));
            T* g = static_cast<T*>(v);
            for (int64_t j = 0; j < A_.nt(); ++j)
                for (int64_t i = 0; i < A_.mt(); ++i) {
                    const Tile<T> t = valid_instance(i, j);
                    copy_tile(g + i * st_.nb + j * st_.nb * ld_, ld_, t.data(), t.stride(), t.mb(), t.nb(), sizeof(T));
                }
            check(slt_xcopy_tri(TypeCode<T>::value, tri == 'U' ? 1 : 0, st_.n, p_, ld_, g, ld_, nullptr));
            slt_device_free(p_);
            p_ = g;
        }
        for (auto& kv : st_.tiles) {
            const int64_t i = kv.first.first, j = kv.first.second;
            auto& node = kv.second;
            auto& home = node.inst.at(node.home);
            if (owned_)
                copy_tile(home.tile.data(), home.tile.stride(), p_ + i * st_.nb + j * st_.nb * ld_, ld_,
                          home.tile.mb(), home.tile.nb(), sizeof(T));
            for (auto& in : node.inst) in.second.state = in.first == node.home ? MOSI::Modified : MOSI::Invalid;
        }
    }
private:
    static MatrixStorage<T>& storage_of(BaseMatrix<T>& A) {
        if (!A.storage()) throw Exception(SLT_ERR_ARG);
        return *A.storage();
    }
    bool all_home_current() const {
        for (const auto& kv : st_.tiles) {
            const auto& node = kv.second;
            auto it = node.inst.find(node.home);
            if (it == node.inst.end() || it->second.state == MOSI::Invalid || it->second.tile.kind() != TileKind::UserOwned)
                return false;
        }
        return int64_t(st_.tiles.size()) == A_.mt() * A_.nt();
    }
    // a valid instance of tile (i, j): the device one when current, else any
    Tile<T> valid_instance(int64_t i, int64_t j) const {
        auto nit = st_.tiles.find({i, j});
        if (nit == st_.tiles.end()) throw Exception(SLT_ERR_ARG);       // missing tile
        const auto& node = nit->second;
        auto d = node.inst.find(0);
        if (d != node.inst.end() && d->second.state != MOSI::Invalid) return d->second.tile;
        for (const auto& in : node.inst)
            if (in.second.state != MOSI::Invalid) return in.second.tile;
        throw Exception(SLT_ERR_ARG);                                   // no valid copy
    }
    BaseMatrix<T>& A_;
    MatrixStorage<T>& st_;
    T* p_ = nullptr;
    int64_t ld_ = 1;
    bool owned_ = false;
};

// Lower-triangular device copy of a Hermitian matrix for the drivers (the
// device layer factors lower triangles): the array itself for Lower, the
// conjugate transpose for Upper, and back.
template <typename T>
class LowerArray {
public:
    explicit LowerArray(HermitianMatrix<T>& A) : d_(A), upper_(A.uplo() == Uplo::Upper), n_(A.n()) {
        if (!upper_) return;
        void* v = nullptr;
        check(slt_device_malloc(sizeof(T) * size_t(n_ > 0 ? n_ : 1) * size_t(n_ > 0 ? n_ : 1), &v));
        t_ = static_cast<T*>(v);
        check(slt_xtranspose(TypeCode<T>::value, n_, n_, d_.data(), d_.ld(), t_, n_ > 0 ? n_ : 1, 1, nullptr));
    }
    ~LowerArray() { if (t_) slt_device_free(t_); }
    LowerArray(const LowerArray&) = delete;
    LowerArray& operator=(const LowerArray&) = delete;
    T* data() const { return upper_ ? t_ : d_.data(); }
    int64_t ld() const { return upper_ ? (n_ > 0 ? n_ : 1) : d_.ld(); }
    void close(bool modified) {
        if (modified && upper_) {
            // back to upper storage through a scratch array, so that only the
            // referenced (upper) triangle of the matrix is written
            void* v = nullptr;
            const int64_t ld = n_ > 0 ? n_ : 1;
            check(slt_device_malloc(sizeof(T) * size_t(ld) * size_t(ld), &v));
            const int rc1 = slt_xtranspose(TypeCode<T>::value, n_, n_, t_, ld, v, ld, 1, nullptr);
            const int rc2 = rc1 ? rc1 : slt_xcopy_tri(TypeCode<T>::value, 1, n_, v, ld, d_.data(), d_.ld(), nullptr);
            slt_device_free(v);
            check(rc2);
        }
        d_.close(modified ? (upper_ ? 'U' : 'L') : 0);
    }
private:
    DeviceArray<T> d_;
    bool upper_;
    int64_t n_;
    T* t_ = nullptr;
};

// RAII device int array for the per-panel pivots
struct DeviceInts {
    int* p = nullptr;
    explicit DeviceInts(int64_t n);
    ~DeviceInts();
};

// Per-type C entry points.
inline int c_getrf(int64_t m, int64_t n, float* A, int64_t ld, int* ip, const slt_options* o, int64_t* info)
{ return slt_sgetrf_device(m, n, A, ld, ip, o, nullptr, info); }
inline int c_getrf(int64_t m, int64_t n, double* A, int64_t ld, int* ip, const slt_options* o, int64_t* info)
{ return slt_dgetrf_device(m, n, A, ld, ip, o, nullptr, info); }
inline int c_getrf(int64_t m, int64_t n, std::complex<float>* A, int64_t ld, int* ip, const slt_options* o,
                   int64_t* info)
{ return slt_cgetrf_device(m, n, A, ld, ip, o, nullptr, info); }
inline int c_getrf(int64_t m, int64_t n, std::complex<double>* A, int64_t ld, int* ip, const slt_options* o,
                   int64_t* info)
{ return slt_zgetrf_device(m, n, A, ld, ip, o, nullptr, info); }

inline int c_getrs(int64_t n, int64_t r, const float* A, int64_t ld, const int* ip, float* B, int64_t ldb,
                   const slt_options* o)
{ return slt_sgetrs_device(n, r, A, ld, ip, B, ldb, o, nullptr); }
inline int c_getrs(int64_t n, int64_t r, const double* A, int64_t ld, const int* ip, double* B, int64_t ldb,
                   const slt_options* o)
{ return slt_dgetrs_device(n, r, A, ld, ip, B, ldb, o, nullptr); }
inline int c_getrs(int64_t n, int64_t r, const std::complex<float>* A, int64_t ld, const int* ip,
                   std::complex<float>* B, int64_t ldb, const slt_options* o)
{ return slt_cgetrs_device('N', n, r, A, ld, ip, B, ldb, o, nullptr); }
inline int c_getrs(int64_t n, int64_t r, const std::complex<double>* A, int64_t ld, const int* ip,
                   std::complex<double>* B, int64_t ldb, const slt_options* o)
{ return slt_zgetrs_device('N', n, r, A, ld, ip, B, ldb, o, nullptr); }

inline int c_potrf(int64_t n, float* A, int64_t ld, const slt_options* o, int64_t* info)
{ return slt_spotrf_device(n, A, ld, o, nullptr, info); }
inline int c_potrf(int64_t n, double* A, int64_t ld, const slt_options* o, int64_t* info)
{ return slt_dpotrf_device(n, A, ld, o, nullptr, info); }
inline int c_potrf(int64_t n, std::complex<float>* A, int64_t ld, const slt_options* o, int64_t* info)
{ return slt_cpotrf_device(n, A, ld, o, nullptr, info); }
inline int c_potrf(int64_t n, std::complex<double>* A, int64_t ld, const slt_options* o, int64_t* info)
{ return slt_zpotrf_device(n, A, ld, o, nullptr, info); }

inline int c_potrs(int64_t n, int64_t r, const float* L, int64_t ld, float* B, int64_t ldb, const slt_options* o)
{ return slt_spotrs_device(n, r, L, ld, B, ldb, o, nullptr); }
inline int c_potrs(int64_t n, int64_t r, const double* L, int64_t ld, double* B, int64_t ldb, const slt_options* o)
{ return slt_dpotrs_device(n, r, L, ld, B, ldb, o, nullptr); }
inline int c_potrs(int64_t n, int64_t r, const std::complex<float>* L, int64_t ld, std::complex<float>* B,
                   int64_t ldb, const slt_options* o)
{ return slt_cpotrs_device(n, r, L, ld, B, ldb, o, nullptr); }
inline int c_potrs(int64_t n, int64_t r, const std::complex<double>* L, int64_t ld, std::complex<double>* B,
                   int64_t ldb, const slt_options* o)
{ return slt_zpotrs_device(n, r, L, ld, B, ldb, o, nullptr); }

}  // namespace detail

// ---- pivots --------------------------------------------------------------------
// The pivot conversion needs the CUDA runtime; it lives in the library.
extern "C" int slt_ipiv_alloc(int64_t n, int** d);
extern "C" int slt_ipiv_free(int* d);
extern "C" int slt_ipiv_download(const int* d, int64_t n, int* h);
extern "C" int slt_ipiv_upload(const int* h, int64_t n, int* d);

inline detail::DeviceInts::DeviceInts(int64_t n) { check(slt_ipiv_alloc(n, &p)); }
inline detail::DeviceInts::~DeviceInts() { slt_ipiv_free(p); }

inline void pivots_from_device(const int* d, int64_t n, int64_t nb, Pivots& pivots)
{
    std::vector<int> h(size_t(n > 0 ? n : 1));
    if (n > 0) check(slt_ipiv_download(d, n, h.data()));
    pivots.assign(size_t((n + nb - 1) / nb), {});
    for (int64_t r = 0; r < n; ++r) pivots[size_t(r / nb)].push_back(Pivot(h[size_t(r)] / nb, h[size_t(r)] % nb));
}

inline void pivots_to_device(const Pivots& pivots, int64_t n, int64_t nb, int* d)
{
    std::vector<int> h(size_t(n > 0 ? n : 1), 0);
    for (int64_t r = 0; r < n; ++r) {
        const Pivot& pv = pivots.at(size_t(r / nb)).at(size_t(r % nb));
        h[size_t(r)] = int(pv.tile_index * nb + pv.element_offset);
    }
    if (n > 0) check(slt_ipiv_upload(h.data(), n, d));
}

// ---- LU (float, double, complex<float>, complex<double>) ---------------------
template <typename T>
int64_t getrf(Matrix<T>& A, Pivots& pivots, const Options& opts = Options())
{
    const int64_t mn = A.m() < A.n() ? A.m() : A.n();
    const int64_t nb = A.storage()->nb;
    detail::DeviceInts piv(mn);
    slt_options o = detail::to_c(opts, nb);
    int64_t info = 0;
    detail::DeviceArray<T> a(A);
    check(detail::c_getrf(A.m(), A.n(), a.data(), a.ld(), piv.p, &o, &info));
    a.close();
    pivots_from_device(piv.p, mn, nb, pivots);
    return info;
}

template <typename T>
void getrs(Matrix<T>& A, Pivots& pivots, Matrix<T>& B, const Options& opts = Options())
{
    const int64_t nb = A.storage()->nb;
    detail::DeviceInts piv(A.n());
    pivots_to_device(pivots, A.n(), nb, piv.p);
    slt_options o = detail::to_c(opts, nb);
    detail::DeviceArray<T> a(A), b(B);
    check(detail::c_getrs(A.n(), B.n(), a.data(), a.ld(), piv.p, b.data(), b.ld(), &o));
    b.close();
}

template <typename T>
int64_t gesv(Matrix<T>& A, Pivots& pivots, Matrix<T>& B, const Options& opts = Options())
{
    const int64_t info = getrf(A, pivots, opts);
    if (info == 0) getrs(A, pivots, B, opts);          // SLATE skips the solve (src/gesv.cc:98-103)
    return info;
}

inline int64_t gesv_mixed(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, Matrix<double>& X, int& iter,
                          const Options& opts = Options())
{
    const int64_t nb = A.storage()->nb;
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, nb);
    int64_t info = 0;
    detail::DeviceArray<double> a(A), b(B), x(X);
    check(slt_dsgesv_device(A.n(), B.n(), a.data(), a.ld(), piv.p, b.data(), b.ld(), x.data(), x.ld(), &o, nullptr,
                            &iter, &info));
    if (iter < 0) a.close();                           // the FP64 fallback left its factors in A
    x.close();
    pivots_from_device(piv.p, A.n(), nb, pivots);
    return info;
}

// gesv_mixed<complex<double>, complex<float>> (zcgesv)
inline int64_t gesv_mixed(Matrix<std::complex<double>>& A, Pivots& pivots, Matrix<std::complex<double>>& B,
                          Matrix<std::complex<double>>& X, int& iter, const Options& opts = Options())
{
    const int64_t nb = A.storage()->nb;
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, nb);
    int64_t info = 0;
    detail::DeviceArray<std::complex<double>> a(A), b(B), x(X);
    check(slt_zcgesv_device(A.n(), B.n(), a.data(), a.ld(), piv.p, b.data(), b.ld(), x.data(), x.ld(), &o, nullptr,
                            &iter, &info));
    if (iter < 0) a.close();
    x.close();
    pivots_from_device(piv.p, A.n(), nb, pivots);
    return info;
}

inline int64_t gesv_mixed_gmres(Matrix<double>& A, Pivots& pivots, Matrix<double>& B, Matrix<double>& X,
                                int& iter, const Options& opts = Options())
{
    const int64_t nb = A.storage()->nb;
    detail::DeviceInts piv(A.n());
    slt_options o = detail::to_c(opts, nb);
    int64_t info = 0;
    detail::DeviceArray<double> a(A), b(B), x(X);
    check(slt_dsgesv_gmres_device(A.n(), B.n(), a.data(), a.ld(), piv.p, b.data(), b.ld(), x.data(), x.ld(), &o,
                                  nullptr, &iter, &info));
    if (iter < 0) a.close();
    x.close();
    pivots_from_device(piv.p, A.n(), nb, pivots);
    return info;
}

// slate::gesv_rbt (src/gesv_rbt.cc): random butterfly transform (Option::Depth,
// default 2), LU without pivoting, FP64 refinement; A receives the factors of
// the transformed matrix.  Returns info.
inline int64_t gesv_rbt(Matrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                        const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    int64_t info = 0;
    detail::DeviceArray<double> a(A), b(B), x(X);
    check(slt_dgesv_rbt_device(A.n(), B.n(), a.data(), a.ld(), b.data(), b.ld(), x.data(), x.ld(), &o, nullptr, &iter,
                               &info));
    a.close();
    x.close();
    return info;
}

inline double gecondest(Norm in_norm, Matrix<double>& A, double Anorm, const Options& opts = Options())
{
    const int64_t nb = A.storage()->nb;
    slt_options o = detail::to_c(opts, nb);
    double rcond = 0.0;
    // the estimate does not depend on the row order: identity pivots
    detail::DeviceInts piv(A.n());
    Pivots id((size_t(A.n()) + size_t(nb) - 1) / size_t(nb));
    for (int64_t r = 0; r < A.n(); ++r) id[size_t(r / nb)].push_back(Pivot(0, r % nb));
    pivots_to_device(id, A.n(), nb, piv.p);
    detail::DeviceArray<double> a(A);
    check(slt_dgecondest_device(char(in_norm), A.n(), a.data(), a.ld(), piv.p, Anorm, &rcond, &o, nullptr));
    return rcond;
}

// ---- Cholesky (lower or upper Hermitian) ---------------------------------------
template <typename T>
int64_t potrf(HermitianMatrix<T>& A, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    int64_t info = 0;
    detail::LowerArray<T> a(A);
    check(detail::c_potrf(A.n(), a.data(), a.ld(), &o, &info));
    a.close(true);
    return info;
}

template <typename T>
void potrs(HermitianMatrix<T>& A, Matrix<T>& B, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    detail::LowerArray<T> a(A);
    detail::DeviceArray<T> b(B);
    check(detail::c_potrs(A.n(), B.n(), a.data(), a.ld(), b.data(), b.ld(), &o));
    b.close();
}

template <typename T>
int64_t posv(HermitianMatrix<T>& A, Matrix<T>& B, const Options& opts = Options())
{
    const int64_t info = potrf(A, opts);
    if (info == 0) potrs(A, B, opts);                  // SLATE skips the solve (src/posv.cc)
    return info;
}

inline int64_t posv_mixed(HermitianMatrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                          const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    int64_t info = 0;
    detail::LowerArray<double> a(A);
    detail::DeviceArray<double> b(B), x(X);
    check(slt_dsposv_device(A.n(), B.n(), a.data(), a.ld(), b.data(), b.ld(), x.data(), x.ld(), &o, nullptr, &iter,
                            &info));
    a.close(iter < 0);
    x.close();
    return info;
}

inline int64_t posv_mixed_gmres(HermitianMatrix<double>& A, Matrix<double>& B, Matrix<double>& X, int& iter,
                                const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    int64_t info = 0;
    detail::LowerArray<double> a(A);
    detail::DeviceArray<double> b(B), x(X);
    check(slt_dsposv_gmres_device(A.n(), B.n(), a.data(), a.ld(), b.data(), b.ld(), x.data(), x.ld(), &o, nullptr,
                                  &iter, &info));
    a.close(iter < 0);
    x.close();
    return info;
}

inline double pocondest(Norm in_norm, HermitianMatrix<double>& A, double Anorm, const Options& opts = Options())
{
    slt_options o = detail::to_c(opts, A.storage()->nb);
    double rcond = 0.0;
    detail::LowerArray<double> a(A);
    check(slt_dpocondest_device(char(in_norm), A.n(), a.data(), a.ld(), Anorm, &rcond, &o, nullptr));
    return rcond;
}

// ---- simplified API (include/slate/simplified_api.hh) -------------------------
template <typename T>
void lu_solve(Matrix<T>& A, Matrix<T>& B, const Options& opts = Options())
{
    Pivots p;
    const int64_t info = gesv(A, p, B, opts);
    if (info != 0) throw Exception(SLT_ERR_ARG);
}
template <typename T>
void lu_factor(Matrix<T>& A, Pivots& pivots, const Options& opts = Options())
{
    getrf(A, pivots, opts);
}
template <typename T>
void lu_solve_using_factor(Matrix<T>& A, Pivots& pivots, Matrix<T>& B, const Options& opts = Options())
{
    getrs(A, pivots, B, opts);
}
template <typename T>
void chol_solve(HermitianMatrix<T>& A, Matrix<T>& B, const Options& opts = Options())
{
    if (posv(A, B, opts) != 0) throw Exception(SLT_ERR_ARG);
}
template <typename T>
void chol_factor(HermitianMatrix<T>& A, const Options& opts = Options())
{
    potrf(A, opts);
}
template <typename T>
void chol_solve_using_factor(HermitianMatrix<T>& A, Matrix<T>& B, const Options& opts = Options())
{
    potrs(A, B, opts);
}

}  // namespace slate_gb300
