// inst_2048.cu -- instantiates the fluid kernels for transform length 2048 (y pass: ny = 2048,
// x pass: nx = 2048) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_2048(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 2048>(d);
    fill_size_kernels<float, 2048>(f);
}
}  // namespace fsibe
