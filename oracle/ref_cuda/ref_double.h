// ref_double.h -- TEST INFRASTRUCTURE, force-included after prelude.h for the
// double-precision host-run build of the reference (libref_sim_f64.so).  The
// reference's dataTypes.h hard-codes PRECISION_SINGLE (dataTypes.h:6); this
// header stands in for it with the same definitions (dataTypes.h:4-38) except
// that ptype is double and PRECISION_DOUBLE is set, which selects the
// reference's own Z2Z branches (fieldslice.cpp:34,46,68,80).  Its include
// guard makes the reference's copy a no-op.
#ifndef DATATYPES_H
#define DATATYPES_H

#include <math.h>

#define PRECISION_DOUBLE
typedef double ptype;

#define BLOCK 256
#define SQRT_BLOCK 8

#define PI 3.14159f

#define EPSILON 0.00001f

typedef ptype fieldPoint;

extern bool verbose;

#include "rts/math/complex.h"
#include "rts/math/vector.h"
#include "rts/math/point.h"
#include "rts/math/quad.h"

typedef rts::complex<ptype> bsComplex;
typedef rts::vector<ptype, 3> bsVector;
typedef rts::point<ptype, 3> bsPoint;
typedef rts::quad<ptype, 3> bsRect;

#endif
