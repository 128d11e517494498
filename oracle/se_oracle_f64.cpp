/* se_oracle_f64.cpp — the FP64 run of the oracle: the same restatement (se_oracle.cpp) compiled
 * with every float turned into a double, for the precision reports of the FP32 / FP16 GPU paths
 * against a double-precision run of the same algorithm. Test infrastructure only.
 *
 * Not double: float literals (1.0f and the like: parameters of the algorithm, already rounded to
 * float in the reference) and the Laine-Karras traversal's bit manipulations (they act on the
 * binary32 image of a coordinate; SO_BITS_FLOAT), so the first-block search makes its discrete
 * decisions at float precision. The C API keeps its names; every float in it is a double, so
 * this library is loaded on its own (linked with -Bsymbolic) and bound with double structs. */
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef float so_binary32_t;
#define SO_BITS_FLOAT so_binary32_t
#define float double

#include "se_oracle.cpp"
