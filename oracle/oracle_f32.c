/* FP32 oracle: reference operation order, quantised voxel storage.
 * TEST INFRASTRUCTURE ONLY (see oracle.h). */
#define OR_F64 0
#include "oracle_impl.h"
