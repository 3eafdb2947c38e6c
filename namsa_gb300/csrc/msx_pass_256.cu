// Multislice pass schedules for lines of length 256 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_256(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<256, 16, 16, 2, 16, 16>>::ops("t16_r16x16"),
    SchedImpl<Sched<256, 32, 8, 2, 8, 8, 4>>::ops("t32_r8x8x4"),
    SchedImpl<Sched<256, 16, 32, 1, 16, 16>>::ops("t16_r16x16_c32"),
    SchedImpl<Sched<256, 32, 16, 1, 8, 8, 4>>::ops("t32_r8x8x4_c16"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
