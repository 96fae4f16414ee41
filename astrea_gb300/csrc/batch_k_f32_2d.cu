// Batched sweep kernels for precision float, 2D.
#include "batch_launch.cuh"
namespace astrea {
template BatchFn<float> get_batched<float, 2>(int, int);
template int get_occupancy<float, 2>(int, int);
}
