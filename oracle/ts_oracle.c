/*
 * CPU oracle: TEST INFRASTRUCTURE ONLY (see ts_oracle.h).  Instantiates the
 * kernel restatement in ts_oracle_body.h for float and for double.
 */
#include <stdlib.h>
#include "ts_oracle.h"

#define real float
#define FN(name) name##_f32
#include "ts_oracle_body.h"
#undef real
#undef FN

#define real double
#define FN(name) name##_f64
#include "ts_oracle_body.h"
#undef real
#undef FN
