// step_fixed_r6w8l.cu -- instantiations of the fixed-point kernel: 6 rows per
// thread, 8 warps per CTA, plane history in shared memory, the next plane
// loaded into registers and the x-1 neighbour read from the history (a
// separate translation unit so that the shapes compile in parallel).
#include "step_fixed.cuh"

namespace fdb {
namespace fx {

void launch_r6w8l(int K, bool in_f64, bool out_f64, int cap, const int64_t* in, int64_t* out,
                  const FixedArgs& a, cudaStream_t st) {
  launch_shape<6, 8, true, 3, kLoadRegs, true>(K, in_f64, out_f64, cap, in, out, a, st);
}

}  // namespace fx
}  // namespace fdb
