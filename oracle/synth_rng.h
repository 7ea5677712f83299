/*
 * Synthetic per-thread uniform stream used by the oracle and by the
 * reference harness when no recorded cuRAND draws are supplied.
 *
 * TEST INFRASTRUCTURE ONLY: the product never uses this stream.  The
 * reference draws `curand_uniform_double(&state[tid])` from 8192 XORWOW
 * states seeded with `curand_init(32, tid, 0, ...)`
 * (src/nucleation2.cu:12-16, :262-263, :315, :342, :392, :421).  That
 * generator lives in the cuRAND device header and only runs on a GPU, so
 * CPU-side parity (oracle vs the reference built for the host) uses this
 * stand-in: a SplitMix64 hash of (seed, tid, counter) mapped to (0, 1],
 * the same half-open range curand_uniform_double returns.  On a GPU the
 * oracle instead consumes draws recorded from cuRAND itself.
 */
#ifndef SEVC_SYNTH_RNG_H
#define SEVC_SYNTH_RNG_H

#include <stdint.h>

static inline uint64_t sevc_synth_mix64(uint64_t z)
{
    /* SplitMix64 finaliser (Steele, Lea, Flood 2014). */
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* k-th draw (k = 0, 1, ...) of stream `tid`: a double in (0, 1]. */
static inline double sevc_synth_uniform(uint64_t seed, uint64_t tid, uint64_t k)
{
    uint64_t z = sevc_synth_mix64(seed ^ sevc_synth_mix64((tid << 32) ^ k));
    return (double)((z >> 11) + 1ull) * (1.0 / 9007199254740992.0);
}

#endif
