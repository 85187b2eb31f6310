// ORACLE cross-check shim — test infrastructure only.
// Compiled by oracle/ref_build.sh together with the reference's own Random.cpp and
// mt/dSFMT.c (taken from the reference tree at build time, never copied into this repo)
// into oracle/_ref/libref_random.so. It exposes the reference's Random:: functions
// (Random.hpp:9-114) through a C ABI so tests/golden/make_golden.py can record their
// outputs as golden vectors for the oracle's restated RNG.
#include <cassert>
#include "Random.hpp"

extern "C" {
void ref_init(int seed) { Random::init(seed); }
double ref_close_open() { return dsfmt_genrand_close_open(&Random::dsfmt); }
double ref_open_open() { return dsfmt_genrand_open_open(&Random::dsfmt); }
double ref_uniform() { return Random::uniform(); }
double ref_uniform0x(double x) { return Random::uniform0x(x); }
double ref_normal() { return Random::normal(); }
double ref_normal_ms(double mu, double sigma) { return Random::normal(mu, sigma); }
void ref_on_dsphere(int dim, double *out) { Random::onDSphere(dim, out); }
}
