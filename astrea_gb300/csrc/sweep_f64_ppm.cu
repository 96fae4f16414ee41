// Sweep kernels for precision double, scheme PPM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<double> get_sweep<double, PPM>(int, int, int, int, int);
}
