// Sweep kernels for precision float, scheme PCM (one translation unit per pair).
#include "sweep_launch.cuh"
namespace astrea {
template SweepFn<float> get_sweep<float, PCM>(int, int, int, int, int);
}
