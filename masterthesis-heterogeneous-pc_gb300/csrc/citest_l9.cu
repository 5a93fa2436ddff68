// Level kernels of levels 9-12 (a translation unit of their own, so that the
// level instantiations compile in parallel).
#include "citest.cuh"

namespace hpc {

void *level_kernel_9_12(int level, bool mixed, bool set) {
  if (mixed && set) {
    switch (level) {
      case 9: return (void *)level_kernel<9, true, kSetOrder>;
      case 10: return (void *)level_kernel<10, true, kSetOrder>;
      case 11: return (void *)level_kernel<11, true, kSetOrder>;
      case 12: return (void *)level_kernel<12, true, kSetOrder>;
      default: return nullptr;
    }
  }
  switch (level) {
    case 9: return mixed ? (void *)level_kernel<9, true> : (void *)level_kernel<9, false>;
    case 10: return mixed ? (void *)level_kernel<10, true> : (void *)level_kernel<10, false>;
    case 11: return mixed ? (void *)level_kernel<11, true> : (void *)level_kernel<11, false>;
    case 12: return mixed ? (void *)level_kernel<12, true> : (void *)level_kernel<12, false>;
    default: return nullptr;
  }
}

}  // namespace hpc
