// C entry point over SLATE's own tile LU panel (slate::tile::getrf,
// src/internal/Tile_getrf.hh:159-447), compiled from the SLATE sources by
// oracle/build_ref.sh into oracle/_ref/ against the stand-in headers in
// oracle/refshim_getrf/ (single-process MPI, loop BLAS, minimal Tile).
// Test infrastructure only: it produces the reference panel pivots and
// factors that pin the oracle's restatement of the panel.
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

#include "internal/Tile_getrf.hh"

namespace {

// internal::getrf_panel<Target::HostTask> on one rank
// (src/internal/internal_getrf.cc:20-121): the panel is a column of tiles of
// height mb (the last one ragged), every tile local; thread_size =
// min(threads, number of tiles) threads each run tile::getrf on the shared
// tile list, and the AuxPivot records become (tile index, offset) pivots.
template <typename T>
int64_t panel(int64_t m, int64_t nb, int64_t mb, T* A, int64_t lda, int64_t ib, int threads, T threshold,
              int64_t* piv_tile, int64_t* piv_off)
{
    using slate::Tile;
    std::vector<Tile<T>> tiles;
    std::vector<int64_t> tile_indices;
    for (int64_t i = 0, r0 = 0; r0 < m; ++i, r0 += mb) {
        tiles.push_back(Tile<T>(std::min(mb, m - r0), nb, A + r0, lda));
        tile_indices.push_back(i);
    }
    if (tiles.empty()) return 0;
    const int64_t diag_len = std::min(tiles[0].mb(), nb);
    const int thread_size = std::max(1, std::min<int>(threads, int(tiles.size())));
    slate::ThreadBarrier barrier;
    std::vector<T> max_value(thread_size);
    std::vector<int64_t> max_index(thread_size), max_offset(thread_size);
    std::vector<T> top_block(size_t(ib) * size_t(nb));
    std::vector<slate::internal::AuxPivot<T>> aux(diag_len);
    int64_t info = 0;
    std::vector<std::thread> ts;
    for (int r = 0; r < thread_size; ++r)
        ts.emplace_back([&, r] {
            slate::tile::getrf(diag_len, ib, tiles, tile_indices, aux, 0, 0, MPI_Comm(0), r, thread_size,
                               barrier, max_value, max_index, max_offset, top_block, threshold, &info);
        });
    for (auto& t : ts) t.join();
    for (int64_t i = 0; i < diag_len; ++i) {
        piv_tile[i] = aux[i].tileIndex();
        piv_off[i] = aux[i].elementOffset();
    }
    return info;
}

// Right-looking LU of an m x n matrix in tiles of nb whose every panel is
// SLATE's tile::getrf (through panel() above); the rest of each step -- the
// panel's row interchanges applied to the columns left and right of it, the
// unit-lower solve of the U12 block row and the trailing update -- is plain
// loops, in the order of impl::getrf (src/getrf.cc:81-236) on one rank.
template <typename T>
int64_t lu(int64_t m, int64_t n, T* A, int64_t lda, int64_t nb, int64_t ib, int threads, T threshold,
           int64_t* piv_tile, int64_t* piv_off)
{
    int64_t info = 0;
    const int64_t mn = std::min(m, n);
    for (int64_t k0 = 0; k0 < mn; k0 += nb) {
        const int64_t kb = std::min(nb, n - k0);
        const int64_t diag = std::min(kb, m - k0);
        T* P = A + k0 + k0 * lda;
        const int64_t pinfo = panel<T>(m - k0, kb, nb, P, lda, ib, threads, threshold, piv_tile + k0, piv_off + k0);
        if (pinfo != 0 && info == 0) info = k0 + pinfo;
        // interchanges on the columns outside the panel, in pivot order
        for (int64_t j = 0; j < diag; ++j) {
            const int64_t r = k0 + piv_tile[k0 + j] * nb + piv_off[k0 + j];
            if (r == k0 + j) continue;
            for (int64_t c = 0; c < n; ++c)
                if (c < k0 || c >= k0 + kb) std::swap(A[k0 + j + c * lda], A[r + c * lda]);
        }
        const int64_t c1 = k0 + kb;
        if (c1 < n) {
            // U12 = L11^{-1} A12 (unit lower), then A22 -= L21 U12
            blas::trsm(blas::Layout::ColMajor, blas::Side::Left, blas::Uplo::Lower, blas::Op::NoTrans,
                       blas::Diag::Unit, diag, n - c1, T(1), P, lda, A + k0 + c1 * lda, lda);
            if (k0 + diag < m)
                blas::gemm(blas::Layout::ColMajor, blas::Op::NoTrans, blas::Op::NoTrans, m - k0 - diag, n - c1,
                           diag, T(-1), A + k0 + diag + k0 * lda, lda, A + k0 + c1 * lda, lda, T(1),
                           A + k0 + diag + c1 * lda, lda);
        }
    }
    return info;
}

} // namespace

extern "C" int64_t ref_getrf_d(int64_t m, int64_t n, double* A, int64_t lda, int64_t nb, int64_t ib, int threads,
                               double threshold, int64_t* piv_tile, int64_t* piv_off)
{
    return lu<double>(m, n, A, lda, nb, ib, threads, threshold, piv_tile, piv_off);
}

extern "C" int64_t ref_getrf_panel_d(int64_t m, int64_t nb, int64_t mb, double* A, int64_t lda, int64_t ib,
                                     int threads, double threshold, int64_t* piv_tile, int64_t* piv_off)
{
    return panel<double>(m, nb, mb, A, lda, ib, threads, threshold, piv_tile, piv_off);
}

extern "C" int64_t ref_getrf_panel_s(int64_t m, int64_t nb, int64_t mb, float* A, int64_t lda, int64_t ib,
                                     int threads, float threshold, int64_t* piv_tile, int64_t* piv_off)
{
    return panel<float>(m, nb, mb, A, lda, ib, threads, threshold, piv_tile, piv_off);
}
