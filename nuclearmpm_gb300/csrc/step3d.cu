#include "mpm_step.cuh"
namespace mpm {
MPM_INSTANTIATE(3)
}
