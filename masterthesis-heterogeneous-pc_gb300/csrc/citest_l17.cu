// The level kernel of levels 17-32: one instantiation with the level read at run time
// (LT = 0: the conditioning-set arrays sized for HPC_MAX_LEVEL members, loops not
// unrolled). Levels this high are reached only by graphs whose neighbour lists stay
// long (skeletons run until no edge has enough neighbours); a translation unit of its
// own so that it compiles in parallel with the unrolled levels.
#include "citest.cuh"

namespace hpc {

void *level_kernel_17_up(int level, bool mixed) {
  if (level < 17 || level > HPC_MAX_LEVEL) return nullptr;
  return mixed ? (void *)level_kernel<0, true> : (void *)level_kernel<0, false>;
}

}  // namespace hpc
