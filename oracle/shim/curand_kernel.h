// Host-only stand-in (oracle reference build only). The reference draws one
// random link per step for its divergence probe; the oracle driver replaces
// that probe with a check of every link, so this generator is never used for
// physics.
#pragma once
typedef unsigned curandState_t;
inline void curand_init(unsigned long long s, int, int, curandState_t *st) { *st = (unsigned)s; }
inline unsigned curand(curandState_t *st) { return *st = *st * 1103515245u + 12345u; }
