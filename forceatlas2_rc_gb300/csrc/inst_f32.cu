// inst_f32.cu -- the FP32 path: every kernel of kernels.cuh instantiated for
// float. Built with FMA contraction and approximate division / square root
// (-ftz=true -prec-div=false -prec-sqrt=false); the steps that must be
// bit-exact use explicit round-to-nearest intrinsics.
#include "batch_impl.cuh"
#include "layout_impl.cuh"

namespace fa2cu {
LayoutBase *make_layout_f32(const fa2_full_params *p, const double *pos, int rep,
                            const LayoutOpts *opts, const EdgeList *edges)
{
    return make_layout<float>(p, pos, rep, opts, edges);
}
double layout_footprint_f32(int n, int ninc, int adjust, int any_fixed, int rep, int sms)
{
    return layout_footprint<float>(n, ninc, adjust, any_fixed, rep, sms);
}
RepulseBase *make_repulse_f32(int device, int n, int adjust, int bh)
{
    return make_repulse<float>(device, n, adjust, bh);
}
BatchBase *make_batch_f32(const fa2_full_params *ps, int count, const double *const *pos,
                          int exact_below, int threads, int npt)
{
    return make_batch<float>(ps, count, pos, exact_below, threads, npt);
}
int tune_batch_f32(int device, int *exact_below, int *threads, int *npt)
{
    return tune_batch<float>(device, exact_below, threads, npt);
}
} // namespace fa2cu
