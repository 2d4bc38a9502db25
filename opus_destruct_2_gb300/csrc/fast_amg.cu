// fast_amg.cu - exact_amg.cu built a second time as the mixed-precision policy's multigrid setup
// (build_hierarchy_fast): FMA contraction allowed and the power iteration's norm a fixed-order
// tree sum (SVXG_FAST_SETUP); see the head of exact_amg.cu.
#define SVXG_FAST_SETUP 1
#include "exact_amg.cu"
