// Sweep kernels for precision float, scheme WENO5 (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<float> get_sweep<float, WENO5>(int, int, int, int, int);
}
