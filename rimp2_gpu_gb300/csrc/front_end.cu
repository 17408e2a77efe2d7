// front_end.cu -- placeholder for the AO->MO transform and metric Cholesky.
#include "common.cuh"
