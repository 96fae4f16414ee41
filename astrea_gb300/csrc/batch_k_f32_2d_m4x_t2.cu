// Batched sweep kernels: float, 2D, model 4 axis 0, 32 x 15 tiles.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(float, 4, 2, 0, 1)
}
