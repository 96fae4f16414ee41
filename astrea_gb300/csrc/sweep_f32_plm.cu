// Sweep kernels for precision float, scheme PLM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<float> get_sweep<float, PLM>(int, int, int, int, int);
}
