// Sweep kernels for precision double, scheme WENO7 (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<double> get_sweep<double, WENO7>(int, int, int, int, int);
}
