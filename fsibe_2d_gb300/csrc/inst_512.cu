// inst_512.cu -- instantiates the fluid kernels for transform length 512 (y pass: ny = 512,
// x pass: nx = 512) in FP64 and FP32.  One translation unit per length keeps builds parallel.
#include "fluid.cuh"

namespace fsibe {
void fill_sizes_512(SizeKernels<double>& d, SizeKernels<float>& f) {
    fill_size_kernels<double, 512>(d);
    fill_size_kernels<float, 512>(f);
}
}  // namespace fsibe
