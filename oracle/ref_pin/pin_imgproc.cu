// Reference-kernel pin module: the image kernels of src/tracking/
// cuda_imgproc.cu -- computeDerivativeK, backProjectDepthK, computeNMapK
// (:217-305) and the headless shading renderSceneK / renderSceneTexturedK
// (:17-108) -- launched by name with the shapes of their host functions
// (8x8 CTAs over the image).
#include "src/tracking/cuda_imgproc.cu"
