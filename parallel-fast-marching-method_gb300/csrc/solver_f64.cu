// solver_f64.cu -- double-precision instantiations of the tile solver
// kernels (sweep and rounds) for every tile shape.
#include "solver.cuh"

namespace fm3dt {

void launch_certify_f64(const CertifyArgs<double> &a, cudaStream_t st)
{
    launch_certify<double>(a, st);
}

void launch_round_f64(int shape, int grid, const RoundArgs<double> &a, cudaStream_t st)
{
#define C_(S) ShapeKernels<double, S>::round(grid, a, st)
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
}

void launch_sweep_f64(int shape, int grid, const SweepArgs<double> &a, cudaStream_t st)
{
#define C_(S) ShapeKernels<double, S>::sweep(grid, a, st)
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
}

int occupancy_round_f64(int shape)
{
    int r = 0;
#define C_(S) r = ShapeKernels<double, S>::occ_round()
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
    return r;
}

int occupancy_sweep_f64(int shape)
{
    int r = 0;
#define C_(S) r = ShapeKernels<double, S>::occ_sweep()
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
    return r;
}

}  // namespace fm3dt

// streaming sweep
#include "stream.cuh"

namespace fm3dt {

void launch_stream_f64(int idx, int grid, const StreamArgs<double> &a, cudaStream_t st)
{
#define C_(X, Z) StreamKernels<double, X, Z>::sweep(grid, a, st)
    FM_STREAM_SWITCH(idx, C_)
#undef C_
}

int occupancy_stream_f64(int idx, bool fresh, bool flow)
{
    int r = 0;
#define C_(X, Z) r = StreamKernels<double, X, Z>::occ(fresh, flow)
    FM_STREAM_SWITCH(idx, C_)
#undef C_
    return r;
}

}  // namespace fm3dt
