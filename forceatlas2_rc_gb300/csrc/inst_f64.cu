// inst_f64.cu -- the FP64 path (precision = "double"): every kernel of
// kernels.cuh instantiated for double, built with -fmad=false and IEEE
// division and square root so that each force is computed with the
// operations, in the order, of the reference's src/forceatlas2.c.
#include "batch_impl.cuh"
#include "layout_impl.cuh"

namespace fa2cu {
LayoutBase *make_layout_f64(const fa2_full_params *p, const double *pos, int rep,
                            const LayoutOpts *opts, const EdgeList *edges)
{
    return make_layout<double>(p, pos, rep, opts, edges);
}
double layout_footprint_f64(int n, int ninc, int adjust, int any_fixed, int rep, int sms)
{
    return layout_footprint<double>(n, ninc, adjust, any_fixed, rep, sms);
}
RepulseBase *make_repulse_f64(int device, int n, int adjust, int bh)
{
    return make_repulse<double>(device, n, adjust, bh);
}
BatchBase *make_batch_f64(const fa2_full_params *ps, int count, const double *const *pos,
                          int exact_below, int threads, int npt)
{
    return make_batch<double>(ps, count, pos, exact_below, threads, npt);
}
int tune_batch_f64(int device, int *exact_below, int *threads, int *npt)
{
    return tune_batch<double>(device, exact_below, threads, npt);
}
} // namespace fa2cu
