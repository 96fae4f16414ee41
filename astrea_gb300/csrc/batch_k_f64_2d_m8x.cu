// Batched sweep kernels: double, 2D, model 8 axis 0.
#include "batch_launch.cuh"
namespace astrea {
ASTREA_BATCH_INST(double, 8, 2, 0, 0)
}
