// inst_256.cu -- instantiates the fluid kernels for transform length 256 (y pass: ny = 256,
// x pass: nx = 256) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_256(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 256>(d);
    fill_size_kernels<float, 256>(f);
}
}  // namespace fsibe
