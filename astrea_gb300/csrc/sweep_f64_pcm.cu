// Sweep kernels for precision double, scheme PCM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<double> get_sweep<double, PCM>(int, int, int, int, int);
}
