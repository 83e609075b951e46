#pragma once
#include "opencv2/cuda_shapes.hpp"
