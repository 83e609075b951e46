/* FP64 oracle: double arithmetic, unquantised voxel storage (error reference).
 * TEST INFRASTRUCTURE ONLY (see oracle.h). */
#define OR_F64 1
#include "oracle_impl.h"
