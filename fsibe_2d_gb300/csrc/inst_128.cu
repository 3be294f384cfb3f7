// inst_128.cu -- instantiates the fluid kernels for transform length 128 (y pass: ny = 128,
// x pass: nx = 128) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_128(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 128>(d);
    fill_size_kernels<float, 128>(f);
}
}  // namespace fsibe
