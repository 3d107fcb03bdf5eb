/* Named by the reference's cmc.h; nothing from it is used on the Henon step
 * (oracle/ref.mk, TEST INFRASTRUCTURE). */
#include "gsl_math.h"
