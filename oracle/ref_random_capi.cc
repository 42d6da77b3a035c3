// C entry points over SLATE's own slate::random::generate (matgen/random.cc),
// compiled from the SLATE sources by oracle/build_ref.sh into oracle/_ref/.
// Used only to produce reference outputs for the oracle's Philox restatement.
#include <cstdint>
#include "random.hh"

extern "C" void ref_generate_d(int dist, int64_t seed, int64_t m, int64_t n,
                               int64_t ioff, int64_t joff, double* A, int64_t lda)
{
    slate::random::generate(slate::random::Dist(dist), seed, m, n, ioff, joff, A, lda);
}

extern "C" void ref_generate_s(int dist, int64_t seed, int64_t m, int64_t n,
                               int64_t ioff, int64_t joff, float* A, int64_t lda)
{
    slate::random::generate(slate::random::Dist(dist), seed, m, n, ioff, joff, A, lda);
}
