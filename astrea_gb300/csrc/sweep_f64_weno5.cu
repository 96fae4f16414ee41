// Sweep kernels for precision double, scheme WENO5 (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<double> get_sweep<double, WENO5>(int, int, int, int, int);
}
