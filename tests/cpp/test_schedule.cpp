// The schedule's round-size rules (rsa_mpi_gb300/csrc/host_common.h), on the host: heuristic_darts, cap_darts,
// class_darts and alive_darts as the single-instance and batched loops chain them.  Exit code 0 when every check
// holds; each failure is printed.
#include <cstdint>
#include <cstdio>

#include "../../rsa_mpi_gb300/csrc/host_common.h"

using namespace rsagpu::host;

static int failures = 0;
#define EXPECT(cond)                                                    \
    do {                                                                \
        if (!(cond)) {                                                  \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);       \
            failures++;                                                 \
        }                                                               \
    } while (0)

// the chain of the heuristic schedule's single-instance loop (proceed)
static uint64_t round_darts(uint64_t V, uint64_t remaining, double class_hit, double alive_ratio) {
    uint64_t C = heuristic_darts(kDefaultFactor, kDefaultMinDarts, kDefaultMaxDarts, V);
    C = cap_darts(C, remaining, kDefaultMinDarts);
    C = class_darts(C, remaining, kDefaultMinDarts, class_hit);
    return alive_darts(C, V, alive_ratio);
}

int main() {
    // the voxel-based size: a quarter dart per voxel, clamped to [4096, 2^26]
    EXPECT(heuristic_darts(0.25, 4096, 1ull << 26, 81746504) == 20436626);
    EXPECT(heuristic_darts(0.25, 4096, 1ull << 26, 100) == 4096);
    EXPECT(heuristic_darts(0.25, 4096, 1ull << 26, 1ull << 30) == (1ull << 26));

    // survivors: the first round of an empty box (every dart survives) is bounded to V/16 darts
    EXPECT(alive_darts(20436626, 81746504, 1.0) == 5109156);
    // ... at the survival ratio of the previous round
    EXPECT(alive_darts(20436626, 81746504, 0.5) == 10218313);
    EXPECT(alive_darts(20436626, 81746504, 0.05) == 20436626);  // few survivors: the voxel size stands
    // ... and never below 2^20 darts (small runs keep their rounds)
    EXPECT(alive_darts(2500000, 10000000, 1.0) == (1u << 20));
    EXPECT(alive_darts(500000, 10000000, 1.0) == 500000);
    EXPECT(alive_darts(4096, 100, 1.0) == 4096);

    // a class with a count: 4x the spheres still wanted in its first round, then 1.25x at the last hit ratio
    EXPECT(class_darts(10445480, 746038, 4096, 0.0) == 2984152);
    EXPECT(class_darts(10445480, 1000000, 4096, 0.25) == 5000000);
    EXPECT(class_darts(10445480, 100, 4096, 0.25) == 4096);         // never below the minimum
    EXPECT(class_darts(10445480, 2000000, 4096, 1e-9) == 10445480);  // hit ratio floored: no division blow-up
    EXPECT(cap_darts(10445480, 100000, 4096) == 1600000);

    // config 2's class (volume fraction 1: about 29.8 M spheres wanted, 11.5 M placed at maximality) is not bounded
    // by its count at the hit ratios its rounds have (the first round: none yet; 5.7 M of 20.4 M darts placed;
    // late rounds: a few per mille): the chain gives the voxel size
    const struct { uint64_t placed; double hit; } rounds[] = {{0, 0.0}, {5697482, 0.28}, {9000000, 0.02},
                                                              {11463514, 0.001}};
    for (const auto& r : rounds) {
        const uint64_t C = round_darts(121811478, 29842552 - r.placed, r.hit, 0.05);
        EXPECT(C == heuristic_darts(kDefaultFactor, kDefaultMinDarts, kDefaultMaxDarts, 121811478));
    }
    // a round is never empty, whatever the inputs
    EXPECT(round_darts(1, 1, 1.0, 1.0) >= 1);
    EXPECT(round_darts(81746504, 0, 0.0, 1.0) >= kDefaultMinDarts);

    if (failures) return 1;
    std::printf("schedule rules: all checks passed\n");
    return 0;
}
