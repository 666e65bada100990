/* Forwarding header of the project-written GSL stand-in (see gsl_shim_core.h). */
#ifndef TF_SHIM_GSL_EIGEN_H
#define TF_SHIM_GSL_EIGEN_H
#include "gsl_shim_core.h"
#endif
