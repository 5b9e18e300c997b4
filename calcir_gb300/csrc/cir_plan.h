// Host-side planning of the batched runners (no CUDA): included by cir_api.cu and compiled
// on its own by the CPU tests.
#pragma once

#include <algorithm>
#include <cmath>

// Chunk length for K steps of St origins, at most kn_max steps a chunk.  The
// tridiagonalisation runs `wave` matrices at a time, and a chunk whose last wave is nearly
// empty pays for about a third of a wave while its few blocks run alone (order 1024 at 456
// resident blocks: 3232 matrices, 7.09 waves, 525 ms; 3168 matrices, 6.95 waves, 501 ms).
// Of the chunkings into as few chunks as kn_max allows, equal in length but the last, the
// one with the least estimated time is taken: whole waves, a part-filled last wave counted
// as at least 0.3 of one; ties go to the longer chunks.
inline int cir_plan_chunk(int K, int St, int kn_max, int wave) {
    kn_max = std::max(1, std::min(kn_max, K));
    wave = std::max(1, wave);
    const int nc = (K + kn_max - 1) / kn_max, kn_min = (K + nc - 1) / nc;
    double best = 1e300;
    int pick = kn_max;
    for (int kn = kn_max; kn >= kn_min; kn--) {
        double cost = 0.0;
        for (int k0 = 0; k0 < K && cost < best; k0 += kn) {
            const double w = (double)St * std::min(kn, K - k0) / wave, f = w - std::floor(w);
            cost += std::floor(w) + (f > 0.0 ? std::max(f, 0.3) : 0.0);
        }
        if (cost < best - 1e-9) {
            best = cost;
            pick = kn;
        }
    }
    return pick;
}

// The first part of a chunk's eigensolver batch split over two streams: whole waves of the
// tridiagonalisation, all but the last one (0: no split, fewer than two waves).
inline int cir_split_first_part(int nmat, int wave) {
    wave = std::max(1, wave);
    return nmat >= 2 * wave ? (nmat / wave - 1) * wave : 0;
}
