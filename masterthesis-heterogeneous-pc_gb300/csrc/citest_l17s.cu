// Set-order kernels of levels 17-24 (citest.cuh), unrolled for their level: the deep
// instances of a batch run until exhausted reach these levels with rows of a few dozen
// neighbours, where the runtime-level kernel of citest_l17.cu (arrays sized for 32
// members, loops not unrolled) spends most of its time in local memory. A translation
// unit of its own so that it compiles in parallel with the other levels.
#include "citest.cuh"

namespace hpc {

void *level_kernel_17_24_set(int level) {
  switch (level) {
    case 17: return (void *)level_kernel<17, true, kSetOrder>;
    case 18: return (void *)level_kernel<18, true, kSetOrder>;
    case 19: return (void *)level_kernel<19, true, kSetOrder>;
    case 20: return (void *)level_kernel<20, true, kSetOrder>;
    case 21: return (void *)level_kernel<21, true, kSetOrder>;
    case 22: return (void *)level_kernel<22, true, kSetOrder>;
    case 23: return (void *)level_kernel<23, true, kSetOrder>;
    case 24: return (void *)level_kernel<24, true, kSetOrder>;
    default: return nullptr;
  }
}

}  // namespace hpc
