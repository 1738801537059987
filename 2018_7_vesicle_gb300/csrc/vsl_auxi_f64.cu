// vsl_auxi_f64.cu -- the FP64 instantiation of the auxiliary level set toolbox and the
// masked integrals (vsl_auxi.cuh), compiled without multiply-add contraction so that it
// rounds like the reference, and the drop-in of auxi_set_calculus_toolbox.
#include "vsl_auxi.cuh"

namespace vsl {

VSL_INSTANTIATE_AUXI(double)

cudaError_t launch_auxi_dropin(AuxOut<double> o, const double *lsf, const double *ahp, AuxFIn<double> fin,
                               const Grid &g, double ds, cudaStream_t s)
{
    k_auxi_dropin<double><<<node_grid(g), dim3(BX, BY), 0, s>>>(o, lsf, ahp, fin, g, ds);
    return cudaGetLastError();
}

}  // namespace vsl
