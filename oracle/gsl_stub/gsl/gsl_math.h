/* Empty stand-in for GSL's gsl_math.h (see gsl_sf_bessel.h in this folder). */
#pragma once
#include <math.h>
