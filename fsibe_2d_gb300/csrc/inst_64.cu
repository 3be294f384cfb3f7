// inst_64.cu -- instantiates the fluid kernels for transform length 64 (y pass: ny = 64,
// x pass: nx = 64) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_64(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 64>(d);
    fill_size_kernels<float, 64>(f);
}
}  // namespace fsibe
