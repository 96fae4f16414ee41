// Batched sweep kernels: double, 2D, model 4 axis 0.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(double, 4, 2, 0, 0)
}
