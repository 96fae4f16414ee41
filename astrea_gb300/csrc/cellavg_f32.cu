// Cell-average pre-pass of the FP32 high-order sweeps (compiled with the FP32 sweeps' flags).
#include "cellavg.cuh"
namespace astrea {
template CellAvgFn<float> get_cell_average<float>(int);
template BatchedCellAvgFn<float> get_batched_cell_average<float>(int);
}
