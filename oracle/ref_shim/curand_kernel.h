/* Test infrastructure for the oracle (never part of the shipped library).
 *
 * Stand-in for <curand_kernel.h> when the reference's render() (Render.cu:28-32,43,...)
 * is compiled as host C++.  cuRAND's XORWOW generator is NVIDIA library code and is not
 * reproduced; both this stand-in and the CUDA kernels of this project draw from PCG32
 * (M. E. O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically Good
 * Algorithms for Random Number Generation", 2014; pcg32_srandom_r / pcg32_random_r):
 *   - curand_init(seed, subsequence, offset, s): stream = subsequence (the pixel offset),
 *     initial state = cpt_ref_seed (the literal seed argument 3317 / 1000*t is replaced
 *     by the seed the harness sets), then `offset` draws are skipped;
 *   - curand_uniform_double(s): one 32-bit draw x mapped to (x + 1) * 2^-32, in (0, 1]
 *     like curand_uniform_double. */
#pragma once
#include <stdint.h>

extern uint64_t cpt_ref_seed;

struct cpt_pcg32_state
{
    uint64_t state;
    uint64_t inc;
};
typedef cpt_pcg32_state curandState;

static inline uint32_t cpt_pcg32_next(curandState* s)
{
    uint64_t old = s->state;
    s->state = old * 6364136223846793005ULL + s->inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
}

static inline void curand_init(unsigned long long seed, unsigned long long subsequence,
                               unsigned long long offset, curandState* s)
{
    (void)seed;
    s->state = 0u;
    s->inc = ((uint64_t)subsequence << 1u) | 1u;
    cpt_pcg32_next(s);
    s->state += cpt_ref_seed;
    cpt_pcg32_next(s);
    for (unsigned long long k = 0; k < offset; ++k) cpt_pcg32_next(s);
}

static inline double curand_uniform_double(curandState* s)
{
    return ((double)cpt_pcg32_next(s) + 1.0) * (1.0 / 4294967296.0);
}
