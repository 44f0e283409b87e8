// solver_f32.cu -- single-precision instantiations of the tile solver
// kernels (sweep and rounds) for every tile shape.
#include "solver.cuh"

namespace fm3dt {

void launch_certify_f32(const CertifyArgs<float> &a, cudaStream_t st)
{
    launch_certify<float>(a, st);
}

void launch_round_f32(int shape, int grid, const RoundArgs<float> &a, cudaStream_t st)
{
#define C_(S) ShapeKernels<float, S>::round(grid, a, st)
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
}

void launch_sweep_f32(int shape, int grid, const SweepArgs<float> &a, cudaStream_t st)
{
#define C_(S) ShapeKernels<float, S>::sweep(grid, a, st)
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
}

int occupancy_round_f32(int shape)
{
    int r = 0;
#define C_(S) r = ShapeKernels<float, S>::occ_round()
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
    return r;
}

int occupancy_sweep_f32(int shape)
{
    int r = 0;
#define C_(S) r = ShapeKernels<float, S>::occ_sweep()
    FM_SHAPE_SWITCH(shape, C_)
#undef C_
    return r;
}

}  // namespace fm3dt

// streaming sweep
#include "stream.cuh"

namespace fm3dt {

void launch_stream_f32(int idx, int grid, const StreamArgs<float> &a, cudaStream_t st)
{
#define C_(X, Z) StreamKernels<float, X, Z>::sweep(grid, a, st)
    FM_STREAM_SWITCH(idx, C_)
#undef C_
}

int occupancy_stream_f32(int idx, bool fresh, bool flow)
{
    int r = 0;
#define C_(X, Z) r = StreamKernels<float, X, Z>::occ(fresh, flow)
    FM_STREAM_SWITCH(idx, C_)
#undef C_
    return r;
}

}  // namespace fm3dt
