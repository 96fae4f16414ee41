// Batched sweep kernels: double, 2D, model 8 axis 1.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(double, 8, 2, 1, 0)
}
