// step_fixed_r4w32.cu -- instantiations of the fixed-point kernel for 4 rows per
// thread and 32 warps per CTA (a separate translation unit so the shapes
// compile in parallel).
#include "step_fixed.cuh"

namespace fdb {
namespace fx {

void launch_r4w32(int K, bool in_f64, bool out_f64, unsigned blocks, const int64_t* in,
                 int64_t* out, const FixedArgs& a, cudaStream_t st) {
  launch_shape<4, 32, 1>(K, in_f64, out_f64, blocks, in, out, a, st);
}

}  // namespace fx
}  // namespace fdb
