// Sweep kernels for precision float, scheme PPM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<float> get_sweep<float, PPM>(int, int, int, int, int);
}
