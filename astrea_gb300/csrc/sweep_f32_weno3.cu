// Sweep kernels for precision float, scheme WENO3 (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<float> get_sweep<float, WENO3>(int, int, int, int, int);
}
