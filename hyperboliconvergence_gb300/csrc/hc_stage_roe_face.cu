// Stage kernels of one interface flux, FP64 and FP32, all tile shapes.
#include "hc_launch.h"

HC_STAGE_INSTANTIATE(FLUX_ROE_FACE)
