// Multislice pass schedules for lines of length 1024 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_1024(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<1024, 32, 8, 1, 32, 32>>::ops("t32_r32x32"),
    SchedImpl<Sched<1024, 32, 8, 1, 16, 8, 8>>::ops("t32_r16x8x8"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
