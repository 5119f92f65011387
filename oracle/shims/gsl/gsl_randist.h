/*
 * Deterministic stand-in for the two GSL random-number calls the reference
 * uses (uniform deviates and Gaussian deviates), so the reference can be
 * compiled as a CPU oracle without GSL.  Test infrastructure only.
 *
 * The reference seeds its generators from the wall clock; this stand-in
 * ignores the requested seed and draws its seed from a process-wide counter
 * (starting at ORACLE_RNG_SEED, default 1), so repeated runs are identical.
 * The generator is splitmix64; Gaussian deviates use the Box-Muller method.
 * Oracle parity never depends on these numbers: initial states for parity
 * runs are loaded from state files.
 */
#ifndef ORACLE_SHIM_GSL_RANDIST_H
#define ORACLE_SHIM_GSL_RANDIST_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct { uint64_t s; int have_spare; double spare; } gsl_rng;
typedef int gsl_rng_type;

static const gsl_rng_type gsl_rng_mt19937_value = 0;
#define gsl_rng_mt19937 (&gsl_rng_mt19937_value)

static inline uint64_t oshim_splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *t)
{
    (void)t;
    gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
    return r;
}

static inline void gsl_rng_set(gsl_rng *r, unsigned long seed)
{
    static uint64_t counter = 0;
    (void)seed;
    const char *env = getenv("ORACLE_RNG_SEED");
    uint64_t base = env ? strtoull(env, NULL, 10) : 1u;
    r->s = base * 0x100000001B3ull + (counter++);
    r->have_spare = 0;
}

static inline void gsl_rng_free(gsl_rng *r) { free(r); }

/* uniform on [0,1) with 53 random bits */
static inline double gsl_rng_uniform(gsl_rng *r)
{
    return (double)(oshim_splitmix64(&r->s) >> 11) * (1.0 / 9007199254740992.0);
}

static inline double gsl_ran_gaussian_ziggurat(gsl_rng *r, double sigma)
{
    if (r->have_spare)
    {
        r->have_spare = 0;
        return sigma * r->spare;
    }
    double u1, u2;
    do { u1 = gsl_rng_uniform(r); } while (u1 <= 0.0);
    u2 = gsl_rng_uniform(r);
    double rad = sqrt(-2.0 * log(u1));
    r->spare = rad * sin(6.283185307179586 * u2);
    r->have_spare = 1;
    return sigma * rad * cos(6.283185307179586 * u2);
}

#endif
