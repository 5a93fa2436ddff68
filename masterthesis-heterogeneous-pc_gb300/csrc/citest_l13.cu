// Level kernels of levels 13-16 (a translation unit of their own, so that the
// level instantiations compile in parallel).
#include "citest.cuh"

namespace hpc {

void *level_kernel_13_16(int level, bool mixed, bool set) {
  if (mixed && set) {
    switch (level) {
      case 13: return (void *)level_kernel<13, true, kSetOrder>;
      case 14: return (void *)level_kernel<14, true, kSetOrder>;
      case 15: return (void *)level_kernel<15, true, kSetOrder>;
      case 16: return (void *)level_kernel<16, true, kSetOrder>;
      default: return nullptr;
    }
  }
  switch (level) {
    case 13: return mixed ? (void *)level_kernel<13, true> : (void *)level_kernel<13, false>;
    case 14: return mixed ? (void *)level_kernel<14, true> : (void *)level_kernel<14, false>;
    case 15: return mixed ? (void *)level_kernel<15, true> : (void *)level_kernel<15, false>;
    case 16: return mixed ? (void *)level_kernel<16, true> : (void *)level_kernel<16, false>;
    default: return nullptr;
  }
}

}  // namespace hpc
