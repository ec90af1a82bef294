// Instantiations of the lifting kernel for one storage type.
#include "launch.cuh"

namespace pgb {

void launch_lift_f32(bool exact, int sched, int R, LiftParams const &p,
                    cudaStream_t s) {
  if (exact) return launch_any<Plain<float, true>, true>(sched, R, p, s);
  return launch_any<Plain<float, false>, false>(-1, R, p, s);
}

} // namespace pgb
