// inst_4096.cu -- instantiates the fluid kernels for transform length 4096 (y pass: ny = 4096,
// x pass: nx = 4096) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_4096(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 4096>(d);
    fill_size_kernels<float, 4096>(f);
}
}  // namespace fsibe
