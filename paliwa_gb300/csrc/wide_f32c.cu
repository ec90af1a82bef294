// Instantiations of the wide lifting kernel (rows of adjacent columns) for
// one storage type.
#include "launch.cuh"

namespace pgb {

void launch_wide_f32c(int sched, int code, LiftParams const &p,
                     cudaStream_t s) {
  launch_wide<RowF32C>(sched, code, p, s);
}

} // namespace pgb
