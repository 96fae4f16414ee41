// Batched sweep kernels: float, 2D, model 4 axis 1.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(float, 4, 2, 1, 0)
}
