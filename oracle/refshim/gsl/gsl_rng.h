/*
 * GSL RNG stand-in for compiling the reference: the generator is a
 * counter-based SplitMix64 stream whose seed comes from the environment
 * variable MTH_REF_SEED (default 1), so runs are reproducible; the
 * reference's own seed (srand(time(NULL)), src/init.c:1008-1011) is ignored.
 */
#ifndef MTH_REFSHIM_GSL_RNG_H
#define MTH_REFSHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char* name; } gsl_rng_type;
typedef struct { unsigned long long seed, counter; } gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
extern unsigned long gsl_rng_default_seed;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* t);
void gsl_rng_free(gsl_rng* r);
double gsl_rng_uniform(gsl_rng* r);
double gsl_rng_uniform_pos(gsl_rng* r);
#ifdef __cplusplus
}
#endif
#endif
