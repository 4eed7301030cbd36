/* usx_oracle_f64.c — double instantiation of the CPU oracle: the FP64 oracle
 * that float errors are reported against (test infrastructure only; see
 * usx_oracle.h). */
#define _GNU_SOURCE
#include <math.h>
#include "usx_oracle.h"

#define R double
#define SFX(name) name##_f64
#define LIT(x) ((double)(x))
#define SQRT sqrt
#define SIN sin
#define COS cos
#define SINCOS sincos
#define POW pow
#define EXP exp
#define ATAN2 atan2
#define TAN tan
#define FLOOR floor
#define CEIL ceil
#define FABS fabs
#define HYPOT hypot
#define LOG10 log10
#define CDIV_WIDE 0
#include "usx_oracle_impl.inc"
