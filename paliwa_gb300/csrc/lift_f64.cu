// Instantiations of the lifting kernel for one storage type.
#include "launch.cuh"

namespace pgb {

void launch_lift_f64(bool exact, int sched, int R, LiftParams const &p,
                    cudaStream_t s) {
  if (exact) return launch_any<Plain<double, true>, true>(sched, R, p, s);
  return launch_any<Plain<double, false>, false>(-1, R, p, s);
}

} // namespace pgb
