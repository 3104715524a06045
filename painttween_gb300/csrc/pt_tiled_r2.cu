// pt_tiled_r2.cu -- tiled patch-distance kernels instantiated for patch radius 2.
#include "pt_energy.cuh"

namespace pt {
cudaError_t launch_tiled_2(int kind, int tm, const Params& P, const TileMaps& M, PatchPlanes work, int arg,
                           uint32_t pass_id, float* out, int wide, cudaStream_t s) {
    return ptk::launch_tiled_r<2>(kind, tm, P, M, work, arg, pass_id, out, wide, s);
}
}  // namespace pt
