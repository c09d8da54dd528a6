/* Oracle build shim (test infrastructure): the reference seeds its sketches with
 * srand(clock()) (Spectral.cpp:120,138).  Linking with -Wl,--wrap=srand routes
 * every such call here, which seeds with a fixed value instead, so the
 * reference's outputs become reproducible.  The seed can be overridden with the
 * environment variable MMSB_REF_SEED. */
#include <stdlib.h>

void __real_srand(unsigned int seed);

void __wrap_srand(unsigned int seed) {
  (void)seed;
  const char* s = getenv("MMSB_REF_SEED");
  __real_srand(s ? (unsigned int)strtoul(s, 0, 10) : 12345u);
}
