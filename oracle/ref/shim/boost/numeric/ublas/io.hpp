// Forwarding header of the project-written uBLAS stand-in.
#include "ublas_shim.hpp"
