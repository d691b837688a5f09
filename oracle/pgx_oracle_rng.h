/* Random stream shared by the oracle, the reference harness and (restated
 * independently in CUDA) the GPU renderer.  TEST INFRASTRUCTURE: only tests,
 * the smoke check and the bench's CPU-baseline leg use anything in oracle/.
 *
 * The reference draws from one std::mt19937 per thread, all seeded 1
 * (Sampling.h:16-23, Renderer.h:260), so its streams are not reproducible
 * per pixel.  Parity runs therefore replace its `Sampler` with this stream:
 * PCG32 (O'Neill 2014: 64-bit LCG, multiplier 6364136223846793005,
 * increment 1442695040888963407, XSH-RR output) whose state is keyed by
 * splitmix64 hashes of (seed, pixel, sample).  A float is the top 24 bits
 * of one output times 2^-24, in [0, 1). */
#ifndef PGX_ORACLE_RNG_H_
#define PGX_ORACLE_RNG_H_

#include <stdint.h>

#define ORC_PCG_MULT 6364136223846793005ULL
#define ORC_PCG_INC 1442695040888963407ULL

static inline uint64_t orc_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

static inline uint64_t orc_pcg_init(uint64_t seed, uint64_t pixel, uint64_t sample) {
    uint64_t key = orc_splitmix64(orc_splitmix64(orc_splitmix64(seed) ^ pixel) ^ sample);
    uint64_t state = ORC_PCG_INC;
    state += key;
    state = state * ORC_PCG_MULT + ORC_PCG_INC;
    return state;
}

static inline uint32_t orc_pcg_next_u32(uint64_t* state) {
    uint64_t old = *state;
    *state = old * ORC_PCG_MULT + ORC_PCG_INC;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
}

static inline float orc_pcg_next_float(uint64_t* state) {
    return (float)(orc_pcg_next_u32(state) >> 8) * (1.0f / 16777216.0f);
}

#endif
