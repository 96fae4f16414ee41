// Sweep kernels for precision double, scheme PLM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<double> get_sweep<double, PLM>(int, int, int, int, int);
}
