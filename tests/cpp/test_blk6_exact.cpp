#include <cstdio>
#include <random>
#include <cstring>
// test_blk6_exact.cpp - the assembly's reduced rigid-block products (atbd_add_rigid_fast) against the
// full loops of blk6::atbd_add (atbd_add_rigid), entry by entry, on the host (-ffp-contract=off).
#include "blk6.cuh"
using namespace svxg;
int main() {
  std::mt19937_64 g(5);
  std::uniform_real_distribution<double> U(-2, 2);
  long bad = 0, tot = 0;
  for (int t = 0; t < 200000; ++t) {
    BondStiffness S;
    for (int i = 0; i < 9; ++i) { S.Dt[i] = U(g) * 1e9; S.Dr[i] = U(g) * 1e8; }
    if (t % 7 == 0) for (int i = 0; i < 9; ++i) if (i % 4) S.Dt[i] = 0.0;  // diagonal D
    V3d ra{U(g), U(g), U(g)}, rb{U(g), U(g), U(g)};
    if (t % 5 == 0) { ra.y = 0; rb.x = 0; }
    double s = (t & 1) ? 1.0 : -1.0;
    double C1[36], C2[36];
    for (int i = 0; i < 36; ++i) C1[i] = C2[i] = (t % 3) ? U(g) * 1e9 : 0.0;
    atbd_add_rigid(ra, S, rb, s, C1);
    atbd_add_rigid_fast(ra, S, rb, s, C2);
    for (int i = 0; i < 36; ++i) { ++tot; if (!(C1[i] == C2[i])) { if (bad < 5) printf("diff t=%d i=%d %.17g %.17g\n", t, i, C1[i], C2[i]); ++bad; } }
  }
  printf("entries %ld, value mismatches %ld\n", tot, bad);
  return bad != 0;
}
