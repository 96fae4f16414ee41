// Batched sweep kernels: float, 1D, model 3 axis 0, model 8 axis 0.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(float, 3, 1, 0, 0)
ASTREA_BATCH_INST(float, 8, 1, 0, 0)
}
