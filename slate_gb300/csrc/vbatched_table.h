// vbatched_table.h -- per-size-bucket choices of the batched solver.
// Written by slate_gb300/tune_vbatched.py from timings on NVIDIA GB300; re-run it
// to regenerate.  For systems with n <= max_n: the panel width of the FP64
// batched factorisation, and for the mixed API the tier (1: FP32 factor +
// FP64 refinement, 0: direct FP64 solve of a copy) and its panel width.
#pragma once

struct VbTune { int max_n; int pb_fp64; int mixed_tier; int pb_mixed; };

static const VbTune kVbTable[] = {
    {64, 16, 1, 16},   // 40000 systems; FP64 pb16/pb32 40.4/43.4 ms; mixed fp32/16 35.9, fp32/32 39.6, fp64/16 42.4 ms
    {128, 16, 1, 16},   // 40000 systems; FP64 pb16/pb32 129.0/142.6 ms; mixed fp32/16 80.6, fp32/32 92.8, fp64/16 137.4 ms
    {256, 16, 1, 16},   // 26986 systems; FP64 pb16/pb32 274.5/298.3 ms; mixed fp32/16 127.4, fp32/32 141.8, fp64/16 296.1 ms
    {512, 16, 1, 16},   // 6764 systems; FP64 pb16/pb32 319.1/329.7 ms; mixed fp32/16 110.4, fp32/32 127.9, fp64/16 340.8 ms
    {1024, 32, 1, 32},   // 1693 systems; FP64 pb16/pb32 496.5/490.3 ms; mixed fp32/16 133.9, fp32/32 121.1, fp64/32 511.6 ms
    {2048, 32, 1, 32},   // 423 systems; FP64 pb16/pb32 936.8/881.4 ms; mixed fp32/16 296.6, fp32/32 248.8, fp64/32 914.4 ms
};
