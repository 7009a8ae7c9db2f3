// Band heights measured by python -m sister_gb300.autotune (no measurements yet: the planner's model decides).
#pragma once
namespace sister {
struct TunedRows {
    int dp, hp_lo, hp_hi, rows;
};
constexpr TunedRows kTunedRows[] = {
    {0, 0, 0, 0}, // end
};
} // namespace sister
