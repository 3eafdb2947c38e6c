// Multislice pass schedules for lines of length 384 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_384(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<384, 16, 16, 2, 8, 8, 6>>::ops("t16_r8x8x6"),
    SchedImpl<Sched<384, 16, 32, 1, 8, 8, 6>>::ops("t16_r8x8x6_c32"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
