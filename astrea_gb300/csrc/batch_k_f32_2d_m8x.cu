// Batched sweep kernels: float, 2D, model 8 axis 0.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(float, 8, 2, 0, 0)
}
