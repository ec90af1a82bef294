// Instantiations of the lifting kernel for one storage type.
#include "launch.cuh"

namespace pgb {

void launch_lift_f32c(bool exact_sym, int sched, int R, LiftParams const &p,
                    cudaStream_t s) {
  if (exact_sym) return launch_any<CompensatedSym, true>(sched, R, p, s);
  return launch_any<Compensated, false>(-1, R, p, s);
}

} // namespace pgb
