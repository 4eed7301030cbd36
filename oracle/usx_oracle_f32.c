/* usx_oracle_f32.c — float instantiation of the CPU oracle (test
 * infrastructure only; see usx_oracle.h). Bit-comparable with the reference's
 * float arithmetic when compiled with -ffp-contract=off. */
#define _GNU_SOURCE
#include <math.h>
#include "usx_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

#define R float
#define SFX(name) name##_f32
#define LIT(x) ((float)(x))
#define SQRT sqrtf
#define SIN sinf
#define COS cosf
#define SINCOS sincosf
#define POW powf
#define EXP expf
#define ATAN2 atan2f
#define TAN tanf
#define FLOOR floorf
#define CEIL ceilf
#define FABS fabsf
#define HYPOT hypotf
#define LOG10 log10f
#define CDIV_WIDE 1
#include "usx_oracle_impl.inc"

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
