// FP32-RHS instantiations of the RHS + stage kernel (state and update stay FP64).
#include "kernels_rhs.cuh"

namespace cns {
int launch_rhs_fp32(int S, int V, const Geom& g, const Phys&, const CoefT<float>& cf, const RhsIn<float>& in,
                    const Update<float>& up, double* scal, int quirk, cudaStream_t s) {
    return launch_rhs_t<float>(S, V, g, cf, in, up, scal, quirk, s);
}
}  // namespace cns
