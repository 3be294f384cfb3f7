// inst_32.cu -- instantiates the fluid kernels for transform length 32 (y pass: ny = 32,
// x pass: nx = 32) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_32(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 32>(d);
    fill_size_kernels<float, 32>(f);
}
}  // namespace fsibe
