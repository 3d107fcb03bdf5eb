/* See hdf5.h beside this file. */
#include "hdf5.h"
