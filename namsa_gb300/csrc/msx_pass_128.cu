// Multislice pass schedules for lines of length 128 (kernels in msx_passes.cuh and msx_tma.cuh).
#include "msx_sched.cuh"

namespace msx {
int schedules_128(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<128, 8, 32, 2, 16, 8>>::ops("t8_r16x8"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
