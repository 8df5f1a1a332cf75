// Stand-in for hipper's CUB alias: hipper::cub is CUB itself on NVIDIA GPUs.
#ifndef NEIGHBOR_REF_HARNESS_HIPPER_CUB_H_
#define NEIGHBOR_REF_HARNESS_HIPPER_CUB_H_
#include <cub/cub.cuh>
namespace hipper
{
namespace cub = ::cub;
}
#endif
