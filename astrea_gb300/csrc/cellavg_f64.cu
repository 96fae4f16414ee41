// Cell-average pre-pass of the FP64 high-order sweeps (compiled without FMA, like the FP64 sweeps).
#include "cellavg.cuh"
namespace astrea {
template CellAvgFn<double> get_cell_average<double>(int);
template BatchedCellAvgFn<double> get_batched_cell_average<double>(int);
}
