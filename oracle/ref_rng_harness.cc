/*
 * Test infrastructure (oracle): prints known-answer streams of the
 * reference's counter-based generator (pbbslib/random.h:38-51, hash64_2 at
 * pbbslib/utilities.h:154-159) and of map_uint64_t (LightNE/PathEmbed.h:25-30)
 * so that the restatements can be pinned against the reference itself.
 *
 *   ref_rng <seed> <fork_index> <count>
 * prints, one per line: the forked state, then <count> lines
 * "rand next_state map_uint64(rand)" along the rand()/next() chain, all
 * integers in decimal and the double in %.17g.
 */
#include "pbbslib/random.h"
#include <cstdio>
#include <cstdlib>

#define TWO63 0x8000000000000000u
#define TWO64f (TWO63*2.0)
static double map_u64(uint64_t u) { double y = (double)u; return y / TWO64f; }

int main(int argc, char** argv) {
  if (argc != 4) { std::fprintf(stderr, "usage: ref_rng seed fork_index count\n"); return 2; }
  size_t seed = std::strtoull(argv[1], nullptr, 10);
  uint64_t idx = std::strtoull(argv[2], nullptr, 10);
  int count = std::atoi(argv[3]);
  pbbs::random r = pbbs::random(seed).fork(idx);
  std::printf("%llu\n", (unsigned long long)r.ith_rand(0));
  for (int i = 0; i < count; ++i) {
    size_t x = r.rand();
    r = r.next();
    std::printf("%llu %llu %.17g\n", (unsigned long long)x,
                (unsigned long long)r.ith_rand(0), map_u64(x));
  }
  return 0;
}
