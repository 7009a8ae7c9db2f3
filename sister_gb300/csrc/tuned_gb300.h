// Generated by python -m sister_gb300.autotune on NVIDIA GB300 (2026-12-04). Do not edit by hand.
// Fastest measured band height of the aggregation per (d-stride, padded height) class; sgm_plan uses it on
// a 152-SM device. Columns: dp, padded height range [lo, hi), rows per band; measured ms of the
// representative rig at the best and at the model's band height in the trailing comment.
#pragma once
namespace sister {
struct TunedRows {
    int dp, hp_lo, hp_hi, rows;
};
constexpr TunedRows kTunedRows[] = {
    {64, 0, 768, 8}, // 480x352x64: 0.724 ms (model R=8: 0.724 ms)
    {64, 768, 1536, 8}, // 1024x768x64: 1.403 ms (model R=8: 1.403 ms)
    {64, 1536, 1073741824, 14}, // 1920x1600x64: 2.813 ms (model R=14: 2.813 ms)
    {128, 0, 768, 8}, // 640x480x128: 1.197 ms (model R=8: 1.197 ms)
    {128, 768, 1536, 10}, // 1280x960x128: 2.073 ms (model R=8: 2.094 ms)
    {128, 1536, 1073741824, 14}, // 2048x1600x128: 3.564 ms (model R=13: 3.588 ms)
    {192, 0, 1024, 8}, // 640x480x192: 1.615 ms (model R=8: 1.615 ms)
    {192, 1024, 1792, 12}, // 1280x1008x192: 2.780 ms (model R=12: 2.780 ms)
    {192, 1792, 1073741824, 14}, // 2048x1600x192: 4.688 ms (model R=14: 4.688 ms)
    {256, 0, 1024, 8}, // 640x480x256: 1.912 ms (model R=8: 1.912 ms)
    {256, 1024, 1792, 12}, // 1920x1080x256: 4.264 ms (model R=12: 4.264 ms)
    {256, 1792, 1073741824, 12}, // 2448x2048x256: 7.263 ms (model R=12: 7.263 ms)
    {384, 0, 1536, 12}, // 1024x720x320: 3.581 ms (model R=12: 3.581 ms)
    {384, 1536, 1073741824, 12}, // 2048x1600x384: 8.235 ms (model R=12: 8.235 ms)
    {512, 0, 2048, 9}, // 1280x960x512: 8.090 ms (model R=9: 8.090 ms)
    {512, 2048, 1073741824, 12}, // 2448x2048x512: 16.849 ms (model R=9: 18.229 ms)
    {0, 0, 0, 0}, // end
};
} // namespace sister
