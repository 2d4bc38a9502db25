// sched_table.h - the row schedule of each kind of BSR operator on GB300: kGroupRow (five rows
// per warp) when the operator's mean blocks per row is at most the kind's bound, else kWarpRow.
// Written by opus_destruct_2_gb300/autotune.py from timings of both schedules on every operator
// of its workloads (the bound that minimizes their summed time); rerun it to refit.
#pragma once

namespace svxg {
// K (FP64), a level's A (FP32), prolongation (FP32), restriction (FP32)
constexpr double kGroupRowMaxMean[4] = {5.789, 5.789, 3.12, 0};
}  // namespace svxg
