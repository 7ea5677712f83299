/*
 * TEST INFRASTRUCTURE ONLY.  Stand-in for the cuRAND device header when
 * the reference is compiled for the CPU by oracle/ref/build_ref.py.
 *
 * curand_init(seed, subsequence, offset, &s) selects stream `subsequence`
 * at position `offset`; curand_uniform_double(&s) returns the next draw of
 * that stream.  Draws come from the synthetic SplitMix64 stream of
 * oracle/synth_rng.h (seed from SEVC_REF_RNG_SEED), or from a table of
 * recorded draws (SEVC_REF_RNG_TABLE: raw doubles, SEVC_REF_RNG_NDRAWS per
 * stream), so that the oracle and the reference consume identical streams.
 */
#ifndef SEVC_FAKE_CURAND_KERNEL_H
#define SEVC_FAKE_CURAND_KERNEL_H

struct curandState { long long tid; long long pos; };

static inline void curand_init(unsigned long long, unsigned long long subsequence,
                               unsigned long long offset, curandState *s)
{
    s->tid = (long long)subsequence;
    s->pos = (long long)offset;
}

double sevc_ref_rng_draw(long long tid, long long pos);

static inline double curand_uniform_double(curandState *s)
{
    return sevc_ref_rng_draw(s->tid, s->pos++);
}

#endif
