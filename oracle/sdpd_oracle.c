/*
 * sdpd_oracle.c — TEST INFRASTRUCTURE.  SDPD oracle in FP64 and FP32
 * (see sp_oracle.h and sdpd_oracle_impl.h).  Compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sp_oracle.h"

#define REAL double
#define SQRT sqrt
#define FABS fabs
#define FMAX fmax
#define SPO_NB spo_nb_f64
#define SPO_FN spo_sdpd_f64
#define SPO_COMP 0
#include "sdpd_oracle_impl.h"
#undef REAL
#undef SQRT
#undef FABS
#undef FMAX
#undef SPO_NB
#undef SPO_FN
#undef SPO_COMP

#define REAL float
#define SQRT sqrtf
#define FABS fabsf
#define FMAX fmaxf
#define SPO_NB spo_nb_f32
#define SPO_FN spo_sdpd_f32
#define SPO_COMP 1
#include "sdpd_oracle_impl.h"
