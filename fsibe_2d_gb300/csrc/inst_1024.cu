// inst_1024.cu -- instantiates the fluid kernels for transform length 1024 (y pass: ny = 1024,
// x pass: nx = 1024) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_1024(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 1024>(d);
    fill_size_kernels<float, 1024>(f);
}
}  // namespace fsibe
