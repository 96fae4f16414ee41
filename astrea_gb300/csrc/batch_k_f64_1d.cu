// Batched sweep kernels for precision double, 1D.
#include "batch_launch.cuh"
namespace astrea {
template BatchFn<double> get_batched<double, 1>(int, int);
template int get_occupancy<double, 1>(int, int);
}
