// Multislice pass schedules for lines of length 384 (kernels in msx_passes.cuh).
#include "msx_passes.cuh"

namespace msx {
int schedules_384(const SchedOps** out) {
  static const SchedOps table[] = {
    SchedImpl<Sched<384, 16, 16, 2, 8, 8, 6>>::ops("t16_r8x8x6"),
  };
  *out = table;
  return (int)(sizeof(table) / sizeof(table[0]));
}
}  // namespace msx
