// Slab kernel instantiations for one arithmetic policy (compiled apart so
// that the library builds in parallel).
#include "slab_launch.cuh"

namespace pgb {
void launch_slab_f32(int sched, SlabParams const &p, cudaStream_t s) {
  launch_slab_any<Plain<float, true>>(sched, p, s);
}
} // namespace pgb
