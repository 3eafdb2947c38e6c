// Multislice pass schedules for lines of length 768 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_768(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<768, 32, 8, 1, 8, 8, 12>>::ops("t32_r8x8x12"),
    SchedImpl<Sched<768, 32, 16, 1, 8, 8, 12>>::ops("t32_r8x8x12_c16"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
