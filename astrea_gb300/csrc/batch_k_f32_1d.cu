// Batched sweep kernels for precision float, 1D.
#include "batch_launch.cuh"
namespace astrea {
template BatchFn<float> get_batched<float, 1>(int, int);
template int get_occupancy<float, 1>(int, int);
}
