// driver_table.h -- per-size-bucket choices of the single-system drivers.
// Written by slate_gb300/tune_drivers.py from timings on NVIDIA GB300; re-run
// it to regenerate.  For a factorisation of order n <= max_n of kind (0 getrf,
// 1 potrf) and update class (0 FP64, 1 FP32 SIMT, 2 tensor cores: TF32 /
// BF16 / FP16 / FP8 / 3xTF32): the SMs given to the panel while the rest of
// the previous step's trailing update runs beside it (0: no overlap) and the
// FP64 update engine (1 DFMA with 64 x 64 tiles, 2 DMMA m16n8k4).  The tile
// size nb stays the caller's (Option::BlockSize): the pivot format of getrf
// and getrs depends on it.
#pragma once

#include <cstdint>

struct DriverTune { int kind; int cls; int64_t max_n; int panel_sms; int engine; };

// Initial values from the lookahead sweep of the GPU (getrf FP64 n = 4096:
// 98.7 ms without overlap, 77.7 with 19 panel SMs; getrf FP32 n = 32768 and
// potrf FP16 n = 65536 faster without overlap).
static const DriverTune kDriverTable[] = {
    {0, 0, int64_t(1) << 62, 19, 1},
    {0, 1, int64_t(1) << 62, 0, 1},
    {0, 2, int64_t(1) << 62, 0, 1},
    {1, 0, int64_t(1) << 62, 19, 1},
    {1, 1, int64_t(1) << 62, 0, 1},
    {1, 2, int64_t(1) << 62, 0, 1},
};
