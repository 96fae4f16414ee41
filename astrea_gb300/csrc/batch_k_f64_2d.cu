// Batched sweep kernels for precision double, 2D.
#include "batch_launch.cuh"
namespace astrea {
template BatchFn<double> get_batched<double, 2>(int, int);
template int get_occupancy<double, 2>(int, int);
}
