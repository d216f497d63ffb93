// roots.cpp -- BFS root selection of the reference driver, restated.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle library).
// cpu_2d/main.cpp:351-392: a default-seeded std::knuth_b feeds
// uniform_int_distribution<int64_t>(0, n-1); a candidate is skipped if it was
// drawn before or if its CSR degree is 0; at most nroots * maxgen draws.
// The engine and distribution are libstdc++'s, so the sequence is the
// reference's on the same standard library.
#include <algorithm>
#include <cstdint>
#include <random>
#include <vector>

#include "g5_oracle.h"

extern "C" int g5o_select_roots(int64_t n, const int64_t *row_off, int nroots,
                                int64_t maxgen, int64_t *roots)
{
    std::knuth_b gen;
    std::uniform_int_distribution<int64_t> dist(0, n - 1);
    std::vector<int64_t> tries;
    int64_t attempts = 0;
    const int64_t maxattempts = (int64_t)nroots * maxgen;
    while ((int)tries.size() < nroots && attempts < maxattempts) {
        ++attempts;
        int64_t s = dist(gen);
        if (std::find(tries.begin(), tries.end(), s) != tries.end()) continue;
        if (row_off[s + 1] - row_off[s] > 0) tries.push_back(s);
    }
    for (size_t i = 0; i < tries.size(); ++i) roots[i] = tries[i];
    return (int)tries.size();
}
