// Multislice pass schedules for lines of length 64 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_64(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<64, 8, 32, 2, 8, 8>>::ops("t8_r8x8"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
