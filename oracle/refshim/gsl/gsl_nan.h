#include "gsl_math.h"
