// Multislice pass schedules for lines of length 512 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_512(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<512, 16, 16, 1, 32, 16>>::ops("t16_r32x16"),
    SchedImpl<Sched<512, 32, 8, 2, 16, 16, 2>>::ops("t32_r16x16x2"),
    SchedImpl<Sched<512, 32, 8, 2, 8, 8, 8>>::ops("t32_r8x8x8"),
    SchedImpl<Sched<512, 32, 16, 1, 16, 16, 2>>::ops("t32_r16x16x2_c16"),
    SchedImpl<Sched<512, 32, 16, 1, 8, 8, 8>>::ops("t32_r8x8x8_c16"),
    SchedImpl<Sched<512, 32, 8, 2, 16, 2, 16>>::ops("t32_r16x2x16"),
    SchedImpl<PairedRow<Sched<512, 32, 8, 2, 16, 2, 16>>>::ops("t32_r16x2x16_pair"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
