// kernels.cuh -- the per-iteration ForceAtlas2 kernels, templated on the
// real type. inst_f32.cu instantiates them for float (FMA contraction, fast
// division and square root: the FP32 path), inst_f64.cu for double with
// -fmad=false and IEEE division (the FP64 path, which keeps the operation
// order of the reference so that it reproduces src/forceatlas2.c).
//
// Steps that must be bit-exact in both precisions (Morton codes, centres of
// mass) use the explicit round-to-nearest intrinsics, which are never fused.
#pragma once

#include "common.cuh"
#include "karras.cuh"
#include "sort_tree.cuh"

namespace fa2cu {

// ---- arithmetic helpers ---------------------------------------------------

__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// Division and square root of the hot loops: approximate in float (2 ulp),
// IEEE in double.
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float fsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double fsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float flog1p(float a) { return log1pf(a); }
__device__ __forceinline__ double flog1p(double a) { return log1p(a); }

// OpenCL min / max of the reference (pipeline.cl), exact.
template <class R> __device__ __forceinline__ R cl_min(R a, R b) { return b < a ? b : a; }
template <class R> __device__ __forceinline__ R cl_max(R a, R b) { return a < b ? b : a; }

template <class R> __device__ __forceinline__ typename RT<R>::R2 mk2(R a, R b)
{
    typename RT<R>::R2 v;
    v.x = a;
    v.y = b;
    return v;
}
template <class R>
__device__ __forceinline__ typename RT<R>::R4 mk4(R a, R b, R c, R d)
{
    typename RT<R>::R4 v;
    v.x = a;
    v.y = b;
    v.z = c;
    v.w = d;
    return v;
}

// Repulsion factor between two nodes (reference src/forceatlas2.c:265-275,
// pipeline.cl:46-55): the force on the first is (xd, yd) * factor.
template <class R, bool ADJUST>
__device__ __forceinline__ R rep_factor(R d2, R mm, R ss, R scaling)
{
    if (ADJUST) {
        const R d = fsqrt(d2) - ss;
        if (d > R(0)) return fdiv(scaling * mm, d * d);
        if (d < R(0)) return R(100) * scaling * mm;
        return R(0);
    }
    return d2 > R(0) ? fdiv(scaling * mm, d2) : R(0);
}

// ---- block reductions -----------------------------------------------------

template <class T> __device__ __forceinline__ T warp_sum(T v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// ---- 1. bounding box (pipeline.cl:61-99) ----------------------------------
// Block partial minima / maxima, then the last block to finish reduces the
// partials: min and max are exact, so the result does not depend on order.
// The end of a bounding-box pass, by every thread of a block with its
// partial minima / maxima: the block's partial, then the last block to
// finish reduces the partials (min and max are exact: the result does not
// depend on order) and writes the box and the Morton quantisation.
template <class R>
__device__ __forceinline__ void bbox_finish(R mnx, R mny, R mxx, R mxy, R *partial, R *bbox,
                                            double *quant, unsigned *ticket)
{
    for (int o = 16; o > 0; o >>= 1) {
        mnx = cl_min(mnx, __shfl_down_sync(0xffffffffu, mnx, o));
        mny = cl_min(mny, __shfl_down_sync(0xffffffffu, mny, o));
        mxx = cl_max(mxx, __shfl_down_sync(0xffffffffu, mxx, o));
        mxy = cl_max(mxy, __shfl_down_sync(0xffffffffu, mxy, o));
    }
    __shared__ R s[4][8];
    __shared__ int last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][w] = mnx;
        s[1][w] = mny;
        s[2][w] = mxx;
        s[3][w] = mxy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 1; k < nw; k++) {
            mnx = cl_min(mnx, s[0][k]);
            mny = cl_min(mny, s[1][k]);
            mxx = cl_max(mxx, s[2][k]);
            mxy = cl_max(mxy, s[3][k]);
        }
        R *o = partial + 4 * blockIdx.x;
        o[0] = mnx;
        o[1] = mny;
        o[2] = mxx;
        o[3] = mxy;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block reduces the partials, every thread a strided share
    __threadfence();
    R a = __ldcg(partial), b = __ldcg(partial + 1), c = __ldcg(partial + 2),
      d = __ldcg(partial + 3);
    for (int k = threadIdx.x; k < (int) gridDim.x; k += blockDim.x) {
        a = cl_min(a, __ldcg(partial + 4 * k));
        b = cl_min(b, __ldcg(partial + 4 * k + 1));
        c = cl_max(c, __ldcg(partial + 4 * k + 2));
        d = cl_max(d, __ldcg(partial + 4 * k + 3));
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = cl_min(a, __shfl_down_sync(0xffffffffu, a, o));
        b = cl_min(b, __shfl_down_sync(0xffffffffu, b, o));
        c = cl_max(c, __shfl_down_sync(0xffffffffu, c, o));
        d = cl_max(d, __shfl_down_sync(0xffffffffu, d, o));
    }
    __syncthreads();
    if (lane == 0) {
        s[0][w] = a;
        s[1][w] = b;
        s[2][w] = c;
        s[3][w] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); k++) {
            a = cl_min(a, s[0][k]);
            b = cl_min(b, s[1][k]);
            c = cl_max(c, s[2][k]);
            d = cl_max(d, s[3][k]);
        }
        bbox[0] = a;
        bbox[1] = b;
        bbox[2] = c;
        bbox[3] = d;
        // the Morton quantisation of pipeline.cl:122-124, in double
        const double w = __dsub_rn((double) c, (double) a), h = __dsub_rn((double) d, (double) b);
        const double extent = cl_max(w, h);
        quant[0] = (double) a;
        quant[1] = (double) b;
        quant[2] = extent > 0.0 ? __ddiv_rn(65535.0, extent) : 0.0;
        // for the float quantisation of k_morton: the scale as a float-float
        // pair (hi, lo) and the minima as floats, 16-byte aligned in slots
        // 4 and 5
        float *qf = reinterpret_cast<float *>(quant + 4);
        qf[0] = (float) quant[2];
        qf[1] = (float) (quant[2] - (double) qf[0]);
        qf[2] = a;
        qf[3] = b;
        *ticket = 0u;
    }
}

template <class R>
__global__ void __launch_bounds__(256)
k_bbox(int n, const typename RT<R>::R2 *__restrict__ pos, R *__restrict__ partial,
       R *__restrict__ bbox, double *__restrict__ quant, unsigned *__restrict__ ticket)
{
    typedef typename RT<R>::R2 R2;
    R mnx, mny, mxx, mxy;
    {
        const R2 p0 = pos[0];
        mnx = mxx = p0.x;
        mny = mxy = p0.y;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const R2 p = pos[i];
        mnx = cl_min(mnx, p.x);
        mny = cl_min(mny, p.y);
        mxx = cl_max(mxx, p.x);
        mxy = cl_max(mxy, p.y);
    }
    bbox_finish<R>(mnx, mny, mxx, mxy, partial, bbox, quant, ticket);
}

// ---- 2. Morton codes (pipeline.cl:105-130) ---------------------------------

__device__ __forceinline__ uint32_t spread16(uint32_t v)
{
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// The quantisation runs in double in both precisions (float coordinates
// widen exactly), so that a layout's tree depends on its positions only, not
// on the precision of the iteration: the FP32 path builds the tree of the
// reference's double construction.
// Quantised coordinate of the Morton code: trunc(clamp((v - min) scale,
// 0, 65535)) with the subtraction and the product rounded in double
// (pipeline.cl:105-130).
__device__ __forceinline__ uint32_t morton_cell(double v, double mn, double scale)
{
    const double f = cl_min(cl_max(__dmul_rn(__dsub_rn(v, mn), scale), 0.0), 65535.0);
    return (uint32_t) f;
}
// The same for a float coordinate, from float arithmetic: the difference
// exactly (TwoSum) and the product with the scale's float-float pair (sh,
// sl) to about 2^-46 relative, i.e. within 1e-9 of the real value, as the
// double computation is within 2e-11. Away from an integer (by 1e-7) and
// from the clamps both truncate alike; the rare others are computed in
// double. (FP64 throughput on this GPU is a small fraction of FP32's.)
__device__ __forceinline__ uint32_t morton_cell(float v, float m, double mn, double scale,
                                                float sh, float sl)
{
    const float d = v - m;                         // TwoSum of v and -m
    const float bv = d - v;
    const float e = (v - (d - bv)) + (-m - bv);    // v - m = d + e exactly
    const float p = d * sh;
    const float pe = fmaf(d, sh, -p);              // d sh = p + pe exactly
    const float lo = fmaf(d, sl, fmaf(e, sh, pe)); // the rest, to 2^-46
    float t = truncf(p);
    float fr = (p - t) + lo;                       // p - t exact below 2^24
    if (fr < 0.0f) {
        t -= 1.0f;
        fr += 1.0f;
    } else if (fr >= 1.0f) {
        t += 1.0f;
        fr -= 1.0f;
    }
    // (a scale below 1e-30 may have a flushed low part: double path)
    if (p > 1.0f && p < 65534.0f && fr > 1e-7f && fr < 1.0f - 1e-7f && sh > 1e-30f)
        return (uint32_t) t;
    return morton_cell((double) v, mn, scale);
}

// Morton codes and the identity order of the nodes (grid-stride). With
// `aux` set, the same launch also makes the sort's digit histograms (its
// histogram pass; the sort then starts with its scatter passes): launch few
// blocks then, as each adds 4 x 256 counts to the global histograms.
template <class R>
__global__ void __launch_bounds__(256)
k_morton(int n, const typename RT<R>::R2 *__restrict__ pos, const double *__restrict__ quant,
         uint32_t *__restrict__ key, uint32_t *__restrict__ idx, uint32_t *__restrict__ aux,
         uint32_t *__restrict__ lookback, size_t nlookback)
{
    __shared__ SortHistShared H;
    pdl_wait();
    if (aux) hist_begin(H, lookback, nlookback); // (uniform)
    const double minx = quant[0], miny = quant[1], scale = quant[2];
    float4 qf = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (sizeof(R) == 4) qf = *reinterpret_cast<const float4 *>(quant + 4);
    // U positions per thread loaded together, then coded
    constexpr int U = 4;
    const int stride = gridDim.x * blockDim.x;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
        typename RT<R>::R2 p[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (i0 + u * stride < n) p[u] = pos[i0 + u * stride];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * stride;
            if (i >= n) break;
            uint32_t cx, cy;
            if constexpr (sizeof(R) == 4) {
                cx = morton_cell(p[u].x, qf.z, minx, scale, qf.x, qf.y);
                cy = morton_cell(p[u].y, qf.w, miny, scale, qf.x, qf.y);
            } else {
                cx = morton_cell(p[u].x, minx, scale);
                cy = morton_cell(p[u].y, miny, scale);
            }
            const uint32_t k = spread16(cx) | (spread16(cy) << 1);
            key[i] = k;
            idx[i] = (uint32_t) i;
            if (aux) hist_add(H, k, 4);
        }
    }
    if (aux) hist_end(H, 4, aux);
}

// ---- 4a. nodes in sorted order and the Karras tree (pipeline.cl:195-270) ----

// The gather and the Karras tree in one launch: thread k writes sorted
// node k's record and builds region k (both read only the sort's output).
template <class R>
__global__ void __launch_bounds__(256)
k_gather_karras(int n, int adjust, const uint32_t *__restrict__ order,
                const typename RT<R>::R2 *__restrict__ pos, const R *__restrict__ mass,
                const R *__restrict__ size, typename RT<R>::R4 *__restrict__ psort,
                const uint32_t *__restrict__ key, int2 *__restrict__ child,
                int2 *__restrict__ range, int *__restrict__ parent, int *__restrict__ rope,
                int *__restrict__ visits, int *__restrict__ status)
{
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    // the node's record is loaded first, so that its scattered loads are in
    // flight during the tree search
    const uint32_t i = order[k];
    const bool ok = i < (uint32_t) n; // always, for a valid sort
    typename RT<R>::R2 p = mk2<R>(R(0), R(0));
    R m = R(0), sz = R(0);
    if (ok) {
        p = pos[i];
        m = mass[i];
        if (adjust) sz = size[i];
    }
    if (k < n - 1) karras_one<true>(k, n, key, child, range, parent, rope, visits);
    if (!ok) atomicOr(status + ST_ERROR, ERR_BOUNDS);
    psort[k] = mk4<R>(p.x, p.y, m, sz);
}

// ---- 4c. bottom-up centres of mass (pipeline.cl:272-323) -------------------
// One thread per leaf climbs the tree; at each region, the first child to
// arrive stops and the second computes the region from both children
// (fixed order a then b: the sums do not depend on who arrives last). No
// thread ever waits. The region's traversal record gets its skip link:
// rope[last] is the right child of the region split just after `last`.

// ---- float-float arithmetic (error-free transformations) ------------------

__device__ __forceinline__ ff2 ff_from(float a) { return ff2{a, 0.0f}; }

// (a.hi + a.lo) + (b.hi + b.lo), renormalised; never fused or reassociated.
__device__ __forceinline__ ff2 ff_add(ff2 a, ff2 b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    return ff2{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

// x * y exactly, as hi + lo (the error term of the product by FMA).
__device__ __forceinline__ ff2 ff_mul(float x, float y)
{
    const float p = __fmul_rn(x, y);
    return ff2{p, __fmaf_rn(x, y, -p)};
}

__device__ __forceinline__ double ff_to_double(ff2 a) { return (double) a.hi + (double) a.lo; }

// ---- per-region sums, in the precision of each path ------------------------

__device__ __forceinline__ Agg<double> leaf_agg(const double4_32a &p)
{
    Agg<double> a;
    a.minx = a.maxx = p.x;
    a.miny = a.maxy = p.y;
    a.m = p.z;
    a.mx = __dmul_rn(p.x, p.z);
    a.my = __dmul_rn(p.y, p.z);
    a.pad = 0.0;
    return a;
}

__device__ __forceinline__ Agg<float> leaf_agg(const float4 &p)
{
    Agg<float> a;
    a.minx = a.maxx = p.x;
    a.miny = a.maxy = p.y;
    a.m = ff_from(p.z);
    a.mx = ff_mul(p.x, p.z);
    a.my = ff_mul(p.y, p.z);
    a.pad = ff2{0.0f, 0.0f};
    return a;
}

__device__ __forceinline__ Agg<double> load_agg_cg(const Agg<double> *a)
{
    Agg<double> v;
    const double2 *p = reinterpret_cast<const double2 *>(a);
    const double2 q0 = __ldcg(p), q1 = __ldcg(p + 1), q2 = __ldcg(p + 2), q3 = __ldcg(p + 3);
    v.minx = q0.x;
    v.miny = q0.y;
    v.maxx = q1.x;
    v.maxy = q1.y;
    v.m = q2.x;
    v.mx = q2.y;
    v.my = q3.x;
    v.pad = 0.0;
    return v;
}

__device__ __forceinline__ Agg<float> load_agg_cg(const Agg<float> *a)
{
    Agg<float> v;
    const float4 *p = reinterpret_cast<const float4 *>(a);
    const float4 q0 = __ldcg(p), q1 = __ldcg(p + 1), q2 = __ldcg(p + 2);
    v.minx = q0.x;
    v.miny = q0.y;
    v.maxx = q0.z;
    v.maxy = q0.w;
    v.m = ff2{q1.x, q1.y};
    v.mx = ff2{q1.z, q1.w};
    v.my = ff2{q2.x, q2.y};
    v.pad = ff2{0.0f, 0.0f};
    return v;
}

// The region from its two children, a then b (the order does not depend on
// which child arrives last).
__device__ __forceinline__ Agg<double> agg_combine(const Agg<double> &a, const Agg<double> &b)
{
    Agg<double> q;
    q.minx = cl_min(a.minx, b.minx);
    q.miny = cl_min(a.miny, b.miny);
    q.maxx = cl_max(a.maxx, b.maxx);
    q.maxy = cl_max(a.maxy, b.maxy);
    q.m = __dadd_rn(a.m, b.m);
    q.mx = __dadd_rn(a.mx, b.mx);
    q.my = __dadd_rn(a.my, b.my);
    q.pad = 0.0;
    return q;
}

__device__ __forceinline__ Agg<float> agg_combine(const Agg<float> &a, const Agg<float> &b)
{
    Agg<float> q;
    q.minx = cl_min(a.minx, b.minx);
    q.miny = cl_min(a.miny, b.miny);
    q.maxx = cl_max(a.maxx, b.maxx);
    q.maxy = cl_max(a.maxy, b.maxy);
    q.m = ff_add(a.m, b.m);
    q.mx = ff_add(a.mx, b.mx);
    q.my = ff_add(a.my, b.my);
    q.pad = ff2{0.0f, 0.0f};
    return q;
}

// (cx, cy, m, size^2) of a region: the reference's finalize
// (pipeline.cl:312-323); in double for the FP64 path, from the float-float
// sums for the FP32 path.
__device__ __forceinline__ double4_32a agg_record(const Agg<double> &q, double /*wscale*/)
{
    const double w = __dsub_rn(q.maxx, q.minx), h = __dsub_rn(q.maxy, q.miny);
    double4_32a c;
    c.x = __ddiv_rn(q.mx, q.m);
    c.y = __ddiv_rn(q.my, q.m);
    c.z = q.m;
    c.w = __dmul_rn(2.0, __dadd_rn(__dmul_rn(w, w), __dmul_rn(h, h)));
    return c;
}

// In float, the record holds w = size^2 * wscale with wscale = (1 + B) /
// theta^2 (B = DECIDE_BAND): the walk's opening test is then d^2 > w, with
// the band of decisions made again in double right below it (region_far).
__device__ __forceinline__ float4 agg_record(const Agg<float> &q, float wscale)
{
    const float m = q.m.hi + q.m.lo;
    const float w = q.maxx - q.minx, h = q.maxy - q.miny;
    return make_float4(__fdiv_rn(q.mx.hi + q.mx.lo, m), __fdiv_rn(q.my.hi + q.my.lo, m), m,
                       2.0f * (w * w + h * h) * wscale);
}

// Arrival at region r: returns the number of children that arrived before
// (0 or 1). acq_rel: the arriving thread's writes are visible before it
// counts, and the second arrival sees the first's. CTA scope when one block
// builds the whole tree (the batched engine), device scope otherwise.
template <bool CTA> __device__ __forceinline__ int arrive(int *v)
{
    int prior;
    if (CTA)
        asm volatile("atom.add.acq_rel.cta.s32 %0, [%1], 1;" : "=r"(prior) : "l"(v) : "memory");
    else
        asm volatile("atom.add.acq_rel.gpu.s32 %0, [%1], 1;" : "=r"(prior) : "l"(v) : "memory");
    return prior;
}

// The climb of leaf k (sorted position) of an n-node tree: every region it
// reaches second gets its sums (agg) and its traversal records.
//
// LOCAL: the block's threads climb from the leaves [s0, s1) (256 P of them),
// so both arrivals at a region whose range lies in [s0, s1) come from this
// block: they count on a shared-memory counter (shv[r - s0]; a Karras region
// r always lies in its own range) at CTA scope, whose release costs a CTA
// fence instead of the device-scope fence of a global counter. Only the
// regions that span two blocks' leaves count on visits[] at device scope.
// The data a second arrival reads (the sibling's sums) was written by the
// thread that arrived first, before its release; which scope the counter has
// changes neither the order of the sums nor the tree.
template <class R, bool CTA, bool LOCAL = false>
__device__ __forceinline__ void climb(int k, int n, const typename RT<R>::R4 *psort,
                                      const int2 *child,
                                      const int *parent,
                                      const int2 *range,
                                      const int *rope, int *visits,
                                      Agg<R> *agg, typename RT<R>::R4 *rec_c, int2 *rec_t,
                                      R wscale, int *status, int *shv = nullptr, int s0 = 0,
                                      int s1 = 0)
{
    const int nl = n - 1;
    int r = parent[nl + k];
    // the sums of the child the thread comes from stay in registers: only
    // the sibling's are loaded
    int prev = nl + k;
    Agg<R> mine = leaf_agg(psort[k]);
    if (LOCAL) {
        // the links of the region above (children, range, parent) are
        // loaded as soon as the region is known, before the arrival there
        // and while the current region's sums are made: one L2 round trip
        // a level less on the chain of the climb
        int2 c = make_int2(-1, -1), rg = make_int2(-1, -1);
        int up = -1;
        if ((unsigned) r < (unsigned) nl) {
            c = child[r];
            rg = range[r];
            up = parent[r];
        }
        for (int depth = 0; r >= 0; depth++) {
            if (r >= nl || depth > 160) {
                atomicOr(status + ST_ERROR, ERR_BOUNDS);
                return;
            }
            const bool here =
                rg.x >= s0 && rg.y < s1 && (unsigned) (r - s0) < (unsigned) (s1 - s0);
            if ((here ? arrive<true>(shv + (r - s0)) : arrive<false>(visits + r)) == 0) return;
            int2 cn = make_int2(-1, -1), rgn = make_int2(-1, -1);
            int upn = -1;
            if ((unsigned) up < (unsigned) nl) {
                cn = child[up];
                rgn = range[up];
                upn = parent[up];
            }
            if (c.x < 0 || c.y < 0 || c.x >= nl + n || c.y >= nl + n || rg.x < 0 ||
                rg.y < 0 || rg.y >= n || (c.x != prev && c.y != prev)) {
                atomicOr(status + ST_ERROR, ERR_BOUNDS);
                return;
            }
            const int2 links =
                make_int2(rg.y - rg.x >= 8 ? c.x : bucket_pack(rg.x, rg.y), rope[rg.y]);
            const bool from_a = c.x == prev;
            const int other = from_a ? c.y : c.x;
            const Agg<R> o =
                other >= nl ? leaf_agg(psort[other - nl]) : load_agg_cg(agg + other);
            const Agg<R> q = from_a ? agg_combine(mine, o) : agg_combine(o, mine);
            agg[r] = q;
            rec_c[r] = agg_record(q, wscale);
            rec_t[r] = links;
            mine = q;
            prev = r;
            r = up;
            c = cn;
            rg = rgn;
            up = upn;
        }
        return;
    }
    // a Karras tree over 32-bit keys and n < 2^27 nodes is < 64 levels deep
    for (int depth = 0; r >= 0; depth++) {
        if (r >= nl || depth > 160) {
            atomicOr(status + ST_ERROR, ERR_BOUNDS);
            return;
        }
        if (arrive<CTA>(visits + r) == 0) return;
        // the region's topology first (its links are known before its sums)
        const int2 c = child[r];
        const int2 rg = range[r];
        if (c.x < 0 || c.y < 0 || c.x >= nl + n || c.y >= nl + n || rg.y < 0 || rg.y >= n ||
            (c.x != prev && c.y != prev)) {
            atomicOr(status + ST_ERROR, ERR_BOUNDS);
            return;
        }
        // a region of at most 8 nodes is never opened: its left link
        // carries its packed range instead (negative)
        const int2 links =
            make_int2(rg.y - rg.x >= 8 ? c.x : bucket_pack(rg.x, rg.y), rope[rg.y]);
        const bool from_a = c.x == prev;
        const int other = from_a ? c.y : c.x;
        const Agg<R> o = other >= nl ? leaf_agg(psort[other - nl]) : load_agg_cg(agg + other);
        // a then b, whichever arrived last
        const Agg<R> q = from_a ? agg_combine(mine, o) : agg_combine(o, mine);
        agg[r] = q;
        rec_c[r] = agg_record(q, wscale);
        rec_t[r] = links;
        mine = q;
        prev = r;
        r = parent[r];
    }
}

template <class R>
__global__ void __launch_bounds__(256)
k_aggregate(int n, const typename RT<R>::R4 *__restrict__ psort,
            const int2 *__restrict__ child, const int *__restrict__ parent,
            const int2 *__restrict__ range, const int *__restrict__ rope,
            int *__restrict__ visits, Agg<R> *__restrict__ agg,
            typename RT<R>::R4 *__restrict__ rec_c, int2 *__restrict__ rec_t, R wscale,
            int *__restrict__ status)
{
    __shared__ int shv[256];
    shv[threadIdx.x] = 0;
    pdl_wait();
    __syncthreads();
    const int s0 = blockIdx.x * 256, s1 = min(s0 + 256, n);
    const int k = s0 + threadIdx.x;
    if (k < n)
        climb<R, false, true>(k, n, psort, child, parent, range, rope, visits, agg, rec_c,
                              rec_t, wscale, status, shv, s0, s1);
}

// The climbs of P leaves per thread, one after the other: with n/P threads
// the launch fits in fewer waves of blocks (1M leaves one per thread are 3.2
// waves of 2048 threads on 152 SMs), and a climb no longer waits for a later
// wave to finish the region above it. CONTIG: thread t takes leaves tP ..
// tP+P-1; else lane l of warp w takes leaves (wP+q)32+l, q < P. Either way a
// block takes the 256 P leaves from 256 P blockIdx.x on, whose inner regions
// count their arrivals in shared memory. Which thread computes a region does
// not change what it computes: the tree is the same. In float the launch
// bound keeps 1536 threads per SM (40 registers: the early-loaded links of
// the next level spill at 32), which the choice of P
// (pick_climb) counts on.
template <class R, int P, bool CONTIG>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 6 : 4)
k_aggregate_multi(int n, const typename RT<R>::R4 *__restrict__ psort,
                  const int2 *__restrict__ child, const int *__restrict__ parent,
                  const int2 *__restrict__ range, const int *__restrict__ rope,
                  int *__restrict__ visits, Agg<R> *__restrict__ agg,
                  typename RT<R>::R4 *__restrict__ rec_c, int2 *__restrict__ rec_t, R wscale,
                  int *__restrict__ status)
{
    __shared__ int shv[256 * P];
#pragma unroll
    for (int q = 0; q < P; q++) shv[q * 256 + threadIdx.x] = 0;
    pdl_wait();
    __syncthreads();
    const int s0 = blockIdx.x * (256 * P), s1 = min(s0 + 256 * P, n);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll 1
    for (int q = 0; q < P; q++) {
        const int k = CONTIG ? t * P + q : ((t >> 5) * P + q) * 32 + (t & 31);
        if (k < n)
            climb<R, false, true>(k, n, psort, child, parent, range, rope, visits, agg, rec_c,
                                  rec_t, wscale, status, shv, s0, s1);
    }
}

// ---- 5. Barnes-Hut traversal (pipeline.cl:329-383) -------------------------
// One thread per node, in sorted order; the walk is stackless: from a region
// the thread goes down to the left child or jumps to the region's skip link,
// which visits the regions in exactly the order of the reference's stack
// (left child first). A small region that is too close is summed node by
// node; each step of the loop handles either one region or one node pair, so
// the threads of a warp stay in step.

// In float, a region whose test d^2 theta^2 > size^2 lands within 1e-4 of
// the boundary is decided again in double, from the region's double sums:
// the float path then approximates exactly the regions the double path
// approximates (a flipped decision would change a node's force by the
// approximation error itself, ~1e-2 of that region's pull).
constexpr float DECIDE_BAND = 1e-4f;

__device__ __forceinline__ float fabs_r(float a) { return fabsf(a); }
__device__ __forceinline__ double fabs_r(double a) { return fabs(a); }

// The rare re-decision of the FP32 walk, in double, from a region's
// float-float sums and float bounding box (exact in double): without
// dividing, d^2 theta^2 > size^2 is (m x - sum m x)^2 + (m y - sum m y)^2
// times theta^2 > size^2 m^2. It agrees with the double construction's test
// except within ~1e-14 of the boundary.
__device__ __forceinline__ bool far_dd(const Agg<float> *a, float xi, float yi, double theta2d)
{
    const float4 *p = reinterpret_cast<const float4 *>(a);
    const float4 box = p[0], q1 = p[1], q2 = p[2];
    const double m = (double) q1.x + (double) q1.y;
    const double mx = (double) q1.z + (double) q1.w;
    const double my = (double) q2.x + (double) q2.y;
    const double w = (double) box.z - (double) box.x, h = (double) box.w - (double) box.y;
    const double s2 = 2.0 * (w * w + h * h);
    const double X = m * (double) xi - mx, Y = m * (double) yi - my;
    return (X * X + Y * Y) * theta2d > s2 * (m * m);
}
__device__ __forceinline__ bool far_dd(const Agg<double> *a, float xi, float yi, double theta2d)
{
    return false; // the FP64 walk decides in double directly
}

// The opening test d^2 theta^2 > size^2 of a region (pipeline.cl:350). The
// FP64 records hold size^2 and the test is made as stated. The FP32 records
// hold w = size^2 (1 + B) / theta^2, the top of the band of relative width B
// around the boundary: a region beyond it is far; one inside the band (d^2
// above w (1 - B) / (1 + B)) is decided again in double; the rest are near.
// (theta = 0: w is infinite, or not a number for a region of size 0, and
// every region is near.)
constexpr float DECIDE_LO = (1.0f - DECIDE_BAND) / (1.0f + DECIDE_BAND);
__device__ __forceinline__ bool region_far(float d2, float w, float /*theta2*/,
                                           const Agg<float> *a, float xi, float yi,
                                           double theta2d)
{
    if (d2 > w) return true;
    if (d2 > w * DECIDE_LO) return far_dd(a, xi, yi, theta2d);
    return false;
}
__device__ __forceinline__ bool region_far(double d2, double w, double theta2,
                                           const Agg<double> *, float, float, double)
{
    return d2 * theta2 > w;
}

// The force of the tree's walk on sorted node k of an n-node tree.
template <class R, bool ADJUST>
__device__ __forceinline__ typename RT<R>::R2
walk(int k, int n, R scaling, R theta2, double theta2d,
     const typename RT<R>::R4 *psort, const typename RT<R>::R4 *rec_c, const int2 *rec_t,
     const Agg<R> *agg, const int *rope, int *status)
{
    typedef typename RT<R>::R4 R4;
    const R4 me = psort[k];
    const R xi = me.x, yi = me.y, mi = me.z, si = me.w;
    R ax = R(0), ay = R(0);
    const int nl = n - 1;
    // walk positions: regions 0 .. nl-1, single nodes nl .. nl+n-1; the walk
    // ends at -1
    const unsigned nend = (unsigned) (nl + n);
    int cur = 0, j = 0, jend = -1;
    // a walk takes at most one step per region (n-1), one per single node
    // reached as a leaf (n) and one per node pair summed (n): more steps than
    // 3n, or a link out of range, is a bug
    const int cap = 3 * n + 64;
    for (int step = 0;; step++) {
        if (j <= jend) {
            if (j != k) {
                const R4 q = psort[j];
                const R xd = xi - q.x, yd = yi - q.y;
                const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi * q.z,
                                                  si + q.w, scaling);
                ax += xd * g;
                ay += yd * g;
            }
            ++j;
            continue;
        }
        if ((unsigned) cur >= nend || step > cap) {
            if (cur != -1) atomicOr(status + ST_ERROR, ERR_BOUNDS);
            break;
        }
        if (cur >= nl) { // a single node
            j = jend = cur - nl;
            cur = rope[j];
            continue;
        }
        const R4 c = rec_c[cur];
        const int2 t = rec_t[cur];
        const R xd = xi - c.x, yd = yi - c.y;
        const R d2 = xd * xd + yd * yd;
        const bool far = region_far(d2, c.w, theta2, agg + cur, (float) xi, (float) yi, theta2d);
        if (far) {
            const R g = fdiv(scaling * (mi * c.z), d2);
            ax += xd * g;
            ay += yd * g;
            cur = t.y;
        } else if (t.x >= 0) {
            cur = t.x;
        } else { // at most 8 nodes: node by node
            j = bucket_first(t.x);
            jend = bucket_last(t.x);
            if (jend >= n) {
                atomicOr(status + ST_ERROR, ERR_BOUNDS);
                break;
            }
            cur = t.y;
        }
    }
    return mk2<R>(ax, ay);
}

template <class R, bool ADJUST, int MINB>
__global__ void __launch_bounds__(256, MINB)
k_traverse(int n, R scaling, R theta2, double theta2d,
           const typename RT<R>::R4 *__restrict__ psort,
           const typename RT<R>::R4 *__restrict__ rec_c, const int2 *__restrict__ rec_t,
           const Agg<R> *__restrict__ agg, const int *__restrict__ rope,
           const uint32_t *__restrict__ order, typename RT<R>::R2 *__restrict__ f,
           int *__restrict__ status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    f[order[k]] = walk<R, ADJUST>(k, n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg,
                                  rope, status);
}

// The walk with its node pairs deferred (FP32 path). In the walk above, a
// warp whose lanes are partly summing node pairs and partly visiting
// regions issues both kinds of step in nearly every iteration. Here the walk
// visits regions only: a small region that is too close (and a single node
// reached as a leaf) is queued as its packed sorted range, and the queued
// node pairs are summed after the walk -- before, if the queue fills up.
// The regions and the pairs are those of walk(); the force is summed in
// another order: the far regions in walk order, then the pairs in walk order.
constexpr int DEFER_QUEUE = 16;

// A node of mass 1 + HEAVY_DEGREE or more (a hub) near equilibrium feels a
// repulsion that nearly cancels an attraction ~100 times larger than the
// net force: summed in plain float, the running sum's roundings reach
// ~1e-4 of the largest net force. The walk adds its terms with Kahan
// compensation for such nodes (in graphs that have any; COMP).
constexpr float HUB_MASS = 1.0f + 128; // 1 + HEAVY_DEGREE (below)

// s += v, compensated when `comp` (c carries the lost low part, negated).
__device__ __forceinline__ void acc_add(float &s, float &c, float v, bool comp)
{
    if (comp) {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    } else {
        s += v;
    }
}
__device__ __forceinline__ void acc_add(double &s, double &, double v, bool) { s += v; }

// Read-only loads of the walk's inputs (non-coherent path in float).
__device__ __forceinline__ float4 ldg_r4(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ double4_32a ldg_r4(const double4_32a *p) { return *p; }

template <class R, bool ADJUST>
__device__ __forceinline__ void sum_pairs(int k, const int *q, int nq, R xi, R yi, R mi, R si,
                                          R scaling, const typename RT<R>::R4 *psort, R &ax,
                                          R &ay, R &cx, R &cy, bool comp)
{
    // one loop over all the queued pairs (bucket after bucket, each in
    // sorted order): the lanes of a warp run as many iterations as the
    // lane with the most pairs, not the most nodes of each bucket in turn
    if (nq <= 0) return;
    int b = 0, j = bucket_first(q[0]), last = bucket_last(q[0]);
    for (;;) {
        if (j != k) {
            const typename RT<R>::R4 p = ldg_r4(psort + j);
            const R xd = xi - p.x, yd = yi - p.y;
            const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi * p.z, si + p.w, scaling);
            acc_add(ax, cx, xd * g, comp);
            acc_add(ay, cy, yd * g, comp);
        }
        if (++j > last) {
            if (++b >= nq) break;
            j = bucket_first(q[b]);
            last = bucket_last(q[b]);
        }
    }
}

template <class R, bool ADJUST, bool COMP = false>
__device__ __forceinline__ typename RT<R>::R2
walk_deferred(int k, int n, R scaling, R theta2, double theta2d,
              const typename RT<R>::R4 *psort, const typename RT<R>::R4 *rec_c,
              const int2 *rec_t, const Agg<R> *agg, const int *rope, int *status)
{
    typedef typename RT<R>::R4 R4;
    const R4 me = psort[k];
    const R xi = me.x, yi = me.y, mi = me.z, si = me.w;
    // a far region's pull is (scaling m_i) m / d^2
    const R smi = scaling * mi;
    R ax = R(0), ay = R(0), cx = R(0), cy = R(0);
    const bool comp = COMP && sizeof(R) == 4 && mi >= R(HUB_MASS);
    const int nl = n - 1;
    const unsigned nend = (unsigned) (nl + n);
    int q[DEFER_QUEUE];
    int nq = 0;
    int cur = 0;
    // one step per region (n - 1) and per single node reached as a leaf
    // (n): at most 2n + 65 steps
    int budget = 2 * n + 65;
    for (;;) {
        // one test a step for the rare cases: a single node, the end of the
        // walk (-1), a link out of range, the step budget spent
        --budget;
        int bucket;
        if (((unsigned) cur >= (unsigned) nl) | (budget < 0)) {
            if ((unsigned) cur >= nend || budget < 0) {
                if (cur != -1) atomicOr(status + ST_ERROR, ERR_BOUNDS);
                break;
            }
            const int j = cur - nl; // a single node
            bucket = bucket_pack(j, j);
            cur = __ldg(rope + j);
        } else {
            const R4 c = ldg_r4(rec_c + cur);
            const int2 t = __ldg(rec_t + cur);
            const R xd = xi - c.x, yd = yi - c.y;
            const R d2 = xd * xd + yd * yd;
            const bool far =
                region_far(d2, c.w, theta2, agg + cur, (float) xi, (float) yi, theta2d);
            if (far) {
                const R g = fdiv(smi * c.z, d2);
                acc_add(ax, cx, xd * g, comp);
                acc_add(ay, cy, yd * g, comp);
                cur = t.y;
                continue;
            }
            if (t.x >= 0) {
                cur = t.x;
                continue;
            }
            if (bucket_last(t.x) >= n) {
                atomicOr(status + ST_ERROR, ERR_BOUNDS);
                break;
            }
            bucket = t.x;
            cur = t.y;
        }
        if (nq == DEFER_QUEUE) {
            sum_pairs<R, ADJUST>(k, q, nq, xi, yi, mi, si, scaling, psort, ax, ay, cx, cy, comp);
            nq = 0;
        }
        q[nq++] = bucket;
    }
    sum_pairs<R, ADJUST>(k, q, nq, xi, yi, mi, si, scaling, psort, ax, ay, cx, cy, comp);
    if (comp) {
        ax -= cx;
        ay -= cy;
    }
    return mk2<R>(ax, ay);
}

template <class R, bool ADJUST, int MINB, bool COMP = false>
__global__ void __launch_bounds__(256, MINB)
k_traverse_deferred(int n, R scaling, R theta2, double theta2d,
                    const typename RT<R>::R4 *__restrict__ psort,
                    const typename RT<R>::R4 *__restrict__ rec_c, const int2 *__restrict__ rec_t,
                    const Agg<R> *__restrict__ agg, const int *__restrict__ rope,
                    const uint32_t *__restrict__ order, typename RT<R>::R2 *__restrict__ f,
                    int *__restrict__ status)
{
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    f[order[k]] = walk_deferred<R, ADJUST, COMP>(k, n, scaling, theta2, theta2d, psort, rec_c,
                                                 rec_t, agg, rope, status);
}

// The walk of P sorted nodes k0 .. k0+cnt-1 (cnt <= P, neighbours in
// Morton order) by one thread. The thread walks the union of the nodes'
// walks, in the same preorder, loading each region once for all of them.
// Each node keeps its own decisions: after it approximates a region, it
// stays inactive until the walk reaches that region's skip link (the first
// region after its subtree), where its own walk would go next; the nodes
// near a small region sum its node pairs together, each skipping itself.
// Every node therefore computes the interactions of its own walk, in the
// same order, with the same arithmetic: the forces are those of walk().
template <class R, bool ADJUST, int P>
__device__ __forceinline__ void
walk_multi(int k0, int cnt, int n, R scaling, R theta2, double theta2d,
           const typename RT<R>::R4 *psort, const typename RT<R>::R4 *rec_c,
           const int2 *rec_t, const Agg<R> *agg, const int *rope, const uint32_t *order,
           typename RT<R>::R2 *f, int *status)
{
    typedef typename RT<R>::R4 R4;
    constexpr int ACTIVE = -2;
    R xi[P], yi[P], mi[P], si[P], ax[P], ay[P];
    int resume[P]; // ACTIVE, or the walk position at which the node resumes
#pragma unroll
    for (int u = 0; u < P; u++) {
        const R4 me = psort[u < cnt ? k0 + u : k0];
        xi[u] = me.x;
        yi[u] = me.y;
        mi[u] = me.z;
        si[u] = me.w;
        ax[u] = ay[u] = R(0);
        resume[u] = u < cnt ? ACTIVE : -1; // a missing node never resumes
    }
    const int nl = n - 1;
    int cur = 0, j = 0, jend = -1;
    unsigned pairs = 0; // nodes summing the current range
    const int cap = 4 * n + 64;
    for (int step = 0;; step++) {
        if (step > cap || cur >= nl + n || jend >= n) {
            atomicOr(status + ST_ERROR, ERR_BOUNDS);
            break;
        }
        if (j <= jend) {
            const R4 q = psort[j];
#pragma unroll
            for (int u = 0; u < P; u++) {
                if (((pairs >> u) & 1u) && j != k0 + u) {
                    const R xd = xi[u] - q.x, yd = yi[u] - q.y;
                    const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi[u] * q.z,
                                                      si[u] + q.w, scaling);
                    ax[u] += xd * g;
                    ay[u] += yd * g;
                }
            }
            ++j;
            continue;
        }
        if (cur < 0) break;
        unsigned act = 0;
#pragma unroll
        for (int u = 0; u < P; u++) {
            if (resume[u] == cur) resume[u] = ACTIVE;
            if (resume[u] == ACTIVE) act |= 1u << u;
        }
        if (cur >= nl) { // a single node
            j = jend = cur - nl;
            pairs = act;
            cur = rope[j];
            continue;
        }
        const R4 c = rec_c[cur];
        const int2 t = rec_t[cur];
        unsigned nearm = 0;
#pragma unroll
        for (int u = 0; u < P; u++) {
            if (!((act >> u) & 1u)) continue;
            const R xd = xi[u] - c.x, yd = yi[u] - c.y;
            const R d2 = xd * xd + yd * yd;
            const bool far =
                region_far(d2, c.w, theta2, agg + cur, (float) xi[u], (float) yi[u], theta2d);
            if (far) {
                const R g = fdiv(scaling * (mi[u] * c.z), d2);
                ax[u] += xd * g;
                ay[u] += yd * g;
                resume[u] = t.y;
            } else {
                nearm |= 1u << u;
            }
        }
        if (nearm == 0) {
            cur = t.y;
        } else if (t.x >= 0) {
            cur = t.x;
        } else {
            j = bucket_first(t.x);
            jend = bucket_last(t.x);
            pairs = nearm;
            cur = t.y;
        }
    }
#pragma unroll
    for (int u = 0; u < P; u++)
        if (u < cnt) f[order[k0 + u]] = mk2<R>(ax[u], ay[u]);
}

template <class R, bool ADJUST, int P>
__global__ void __launch_bounds__(256)
k_traverse_multi(int n, R scaling, R theta2, double theta2d,
                 const typename RT<R>::R4 *__restrict__ psort,
                 const typename RT<R>::R4 *__restrict__ rec_c,
                 const int2 *__restrict__ rec_t, const Agg<R> *__restrict__ agg,
                 const int *__restrict__ rope, const uint32_t *__restrict__ order,
                 typename RT<R>::R2 *__restrict__ f, int *__restrict__ status)
{
    const int k0 = (blockIdx.x * blockDim.x + threadIdx.x) * P;
    if (k0 >= n) return;
    walk_multi<R, ADJUST, P>(k0, min(P, n - k0), n, scaling, theta2, theta2d, psort, rec_c,
                             rec_t, agg, rope, order, f, status);
}

// The same walk, warp-synchronous. The 32 threads of a warp (neighbours in
// Morton order) walk the tree together, one region per step, so that every
// load is a broadcast and no branch diverges; a region is opened when any
// lane needs it opened. Each lane keeps its own decisions: after it
// approximates a region (or sums its small range), the lane stays inactive
// until the walk reaches the first region past that region's subtree --
// in preorder the first region whose first sorted node is `last + 1`. A lane
// therefore computes exactly the interactions of the per-thread walk, in the
// same order, with the same arithmetic: the forces are identical.
template <class R, bool ADJUST>
__global__ void __launch_bounds__(256)
k_traverse_warp(int n, R scaling, R theta2, double theta2d,
                const typename RT<R>::R4 *__restrict__ psort,
                const typename RT<R>::R4 *__restrict__ rec_c,
                const int2 *__restrict__ rec_t, const int2 *__restrict__ range,
                const Agg<R> *__restrict__ agg, const int *__restrict__ rope,
                const uint32_t *__restrict__ order, typename RT<R>::R2 *__restrict__ f,
                int *__restrict__ status)
{
    typedef typename RT<R>::R4 R4;
    const unsigned FULL = 0xffffffffu;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if ((k & ~31) >= n) return; // whole warp past the end
    const bool valid = k < n;
    const R4 me = psort[valid ? k : n - 1];
    const R xi = me.x, yi = me.y, mi = me.z, si = me.w;
    R ax = R(0), ay = R(0);
    const int nl = n - 1;
    // active while the current region's first sorted node is >= resume
    int resume = valid ? 0 : 0x7fffffff;
    int cur = 0; // uniform across the warp
    const int cap = 2 * n + 64;
    for (int step = 0; cur >= 0; step++) {
        if (step > cap || cur >= nl + n) { // uniform
            if ((threadIdx.x & 31) == 0) atomicOr(status + ST_ERROR, ERR_BOUNDS);
            break;
        }
        if (cur >= nl) { // a single node
            const int j = cur - nl;
            if (j >= resume && j != k) {
                const R4 q = psort[j];
                const R xd = xi - q.x, yd = yi - q.y;
                const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi * q.z, si + q.w,
                                                  scaling);
                ax += xd * g;
                ay += yd * g;
            }
            cur = rope[j];
            continue;
        }
        const R4 c = rec_c[cur];
        const int2 t = rec_t[cur];
        const int2 rg = range[cur]; // first, last
        bool open = false, direct = false;
        if (rg.x >= resume) {
            const R xd = xi - c.x, yd = yi - c.y;
            const R d2 = xd * xd + yd * yd;
            const bool far =
                region_far(d2, c.w, theta2, agg + cur, (float) xi, (float) yi, theta2d);
            if (far) {
                const R g = fdiv(scaling * (mi * c.z), d2);
                ax += xd * g;
                ay += yd * g;
                resume = rg.y + 1;
            } else if (t.x >= 0) {
                open = true;
            } else {
                direct = true;
                resume = rg.y + 1;
            }
        }
        if (__any_sync(FULL, direct)) {
            for (int j = rg.x; j <= rg.y; j++) {
                const R4 q = psort[j];
                if (direct && j != k) {
                    const R xd = xi - q.x, yd = yi - q.y;
                    const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi * q.z, si + q.w,
                                                      scaling);
                    ax += xd * g;
                    ay += yd * g;
                }
            }
        }
        cur = __any_sync(FULL, open) ? t.x : t.y;
    }
    if (valid) f[order[k]] = mk2<R>(ax, ay);
}

// Instrumented copy of the walk: counts regions visited and node pairs
// computed (for the traffic estimate of the roofline; never timed).
template <class R>
__global__ void __launch_bounds__(256)
k_traverse_count(int n, R theta2, double theta2d, const typename RT<R>::R4 *__restrict__ psort,
                 const typename RT<R>::R4 *__restrict__ rec_c,
                 const int2 *__restrict__ rec_t, const Agg<R> *__restrict__ agg,
                 const int *__restrict__ rope, unsigned long long *__restrict__ counts)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long visits = 0, pairs = 0;
    if (k < n) {
        const typename RT<R>::R4 me = psort[k];
        const int nl = n - 1;
        int cur = 0;
        for (int step = 0; cur >= 0 && cur < nl + n && step <= 4 * n + 64; step++) {
            if (cur >= nl) {
                pairs += (cur - nl != k);
                cur = rope[cur - nl];
                continue;
            }
            ++visits;
            const typename RT<R>::R4 c = rec_c[cur];
            const int2 t = rec_t[cur];
            const R xd = me.x - c.x, yd = me.y - c.y;
            const R d2 = xd * xd + yd * yd;
            const bool far =
                region_far(d2, c.w, theta2, agg + cur, (float) me.x, (float) me.y, theta2d);
            if (far) {
                cur = t.y;
            } else if (t.x >= 0) {
                cur = t.x;
            } else {
                const int first = bucket_first(t.x), last = bucket_last(t.x);
                pairs += last - first + 1 - (k >= first && k <= last);
                cur = t.y;
            }
        }
    }
    visits = warp_sum(visits);
    pairs = warp_sum(pairs);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts, visits);
        atomicAdd(counts + 1, pairs);
    }
}

// ---- 6. gravity and attraction (pipeline.cl:389-429) -----------------------

// Nodes of at least this many incidences (hubs of scale-free graphs) are
// summed by a warp each in the FP32 path (k_attract_heavy, launched before
// the attraction): one thread looping over a hub's thousands of incidences
// would hold up its whole launch. The FP64 path keeps one thread per node:
// its sums follow the reference's edge order.
constexpr int HEAVY_DEGREE = 128;
static_assert(HUB_MASS == 1.0f + HEAVY_DEGREE, "hubs of the walk and of the attraction");

// Gravity and attraction on node i of a graph whose arrays start at pos,
// mass, size (node indices of inc are relative to them), added to the
// repulsion already in f[i]. SKIP_HEAVY: a node of HEAVY_DEGREE incidences
// or more gets its gravity only (k_attract_heavy added its attraction).
// An incidence, read once per iteration: streamed (evict first), so that the
// ~100 MB of incidence lists do not push the positions the attraction
// gathers out of L2.
__device__ __forceinline__ Inc<float> load_inc(const Inc<float> *p)
{
    const int2 v = __ldcs(reinterpret_cast<const int2 *>(p));
    Inc<float> c;
    c.j = v.x;
    c.coef = __int_as_float(v.y);
    return c;
}
__device__ __forceinline__ Inc<double> load_inc(const Inc<double> *p) { return *p; }

//
// OWN (FP32, the attraction run beside the walk): f is the attraction's own
// buffer, and the sum starts at 0 -- at a hub's incidence sum, which
// k_attract_heavy<R, true> wrote there.
template <class R, bool SKIP_HEAVY = false, bool OWN = false>
__device__ __forceinline__ void attract_one(int i, R gravity, int strong, int linlog, int adjust,
                                            const typename RT<R>::R2 *pos,
                                            const R *mass,
                                            const R *size,
                                            const int *off,
                                            const Inc<R> *inc,
                                            typename RT<R>::R2 *f)
{
    const typename RT<R>::R2 p = pos[i];
    const R xi = p.x, yi = p.y;
    R ax = R(0), ay = R(0);
    if (!OWN || (SKIP_HEAVY && off[i + 1] - off[i] >= HEAVY_DEGREE)) {
        const typename RT<R>::R2 a = f[i];
        ax = a.x;
        ay = a.y;
    }
    if (gravity != R(0)) {
        const R dist = fsqrt(xi * xi + yi * yi);
        if (dist > R(0)) {
            const R g = strong ? gravity * mass[i] : fdiv(gravity * mass[i], dist);
            ax -= xi * g;
            ay -= yi * g;
        }
    }
    const R si = adjust ? size[i] : R(0);
    const int e1 = off[i + 1];
    if (SKIP_HEAVY && e1 - off[i] >= HEAVY_DEGREE) {
        f[i] = mk2<R>(ax, ay);
        return;
    }
    // incidences in edge order; the loads of four are issued before any of
    // their neighbours' positions is needed (memory-level parallelism), and
    // the sum keeps the order
    constexpr int U = 4;
    for (int e0 = off[i]; e0 < e1; e0 += U) {
        Inc<R> c[U];
        typename RT<R>::R2 q[U];
#pragma unroll
        for (int u = 0; u < U; u++) c[u] = load_inc(inc + (e0 + u < e1 ? e0 + u : e0));
#pragma unroll
        for (int u = 0; u < U; u++) q[u] = pos[c[u].j];
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (e0 + u >= e1) break;
            const R xd = xi - q[u].x, yd = yi - q[u].y;
            R g = -c[u].coef;
            if (adjust || linlog) {
                R dist = fsqrt(xd * xd + yd * yd);
                if (adjust) dist -= si + size[c[u].j];
                if (!(dist > R(0))) continue;
                if (linlog) g *= fdiv(flog1p(dist), dist);
            }
            ax += xd * g;
            ay += yd * g;
        }
    }
    f[i] = mk2<R>(ax, ay);
}

template <class R>
__global__ void __launch_bounds__(256)
k_attract(int n, R gravity, int strong, int linlog, int adjust,
          const typename RT<R>::R2 *__restrict__ pos, const R *__restrict__ mass,
          const R *__restrict__ size, const int *__restrict__ off,
          const Inc<R> *__restrict__ inc, typename RT<R>::R2 *__restrict__ f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        attract_one<R, sizeof(R) == 4>(i, gravity, strong, linlog, adjust, pos, mass, size, off,
                                       inc, f);
}

// The nodes of HEAVY_DEGREE incidences or more (any order: each is summed
// on its own). `list` holds room for ninc / HEAVY_DEGREE of them, and its
// count after them.
static __global__ void __launch_bounds__(256)
k_heavy_list(int n, const int *__restrict__ off, int *__restrict__ list, int cap)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || off[i + 1] - off[i] < HEAVY_DEGREE) return;
    const int k = atomicAdd(list + cap, 1);
    if (k < cap) list[k] = i;
}

// The attraction of the heavy nodes (FP32 path), one warp per node, added to
// the repulsion in f: lane l sums incidences l, l + 32, ... in order, then
// the lanes' sums are added pairwise across lane distances 16, 8, 4, 2, 1
// (every lane ends with the same total). Gravity follows in the attraction
// launch.
// SET (the attraction run beside the walk): the sum is written to f, the
// attraction's own buffer, instead of added to the repulsion there.
template <class R, bool SET = false>
__global__ void __launch_bounds__(256)
k_attract_heavy(int nheavy, const int *__restrict__ list, int linlog, int adjust,
                const typename RT<R>::R2 *__restrict__ pos, const R *__restrict__ size,
                const int *__restrict__ off, const Inc<R> *__restrict__ inc,
                typename RT<R>::R2 *__restrict__ f)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nheavy) return; // the whole warp
    const int i = list[w];
    const typename RT<R>::R2 p = pos[i];
    const R xi = p.x, yi = p.y;
    const R si = adjust ? size[i] : R(0);
    const int e1 = off[i + 1];
    R ax = R(0), ay = R(0);
    for (int e = off[i] + lane; e < e1; e += 32) {
        const Inc<R> c = inc[e];
        const typename RT<R>::R2 q = pos[c.j];
        const R xd = xi - q.x, yd = yi - q.y;
        R g = -c.coef;
        if (adjust || linlog) {
            R dist = fsqrt(xd * xd + yd * yd);
            if (adjust) dist -= si + size[c.j];
            if (!(dist > R(0))) continue;
            if (linlog) g *= fdiv(flog1p(dist), dist);
        }
        ax += xd * g;
        ay += yd * g;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, o);
        ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    if (lane == 0) {
        if (SET) {
            f[i] = mk2<R>(ax, ay);
        } else {
            const typename RT<R>::R2 a = f[i];
            f[i] = mk2<R>(a.x + ax, a.y + ay);
        }
    }
}

// Gravity and attraction of every node into the attraction's own buffer fa
// (FP32, run on a second stream beside the tree build and the walk):
// grid-stride over the nodes with a grid of a few blocks per SM, so that
// the walk keeps most of every SM. k_join_swing adds fa to the repulsion.
template <class R>
__global__ void __launch_bounds__(256)
k_attract_own(int n, R gravity, int strong, int linlog, int adjust,
              const typename RT<R>::R2 *__restrict__ pos, const R *__restrict__ mass,
              const R *__restrict__ size, const int *__restrict__ off,
              const Inc<R> *__restrict__ inc, typename RT<R>::R2 *__restrict__ fa)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        attract_one<R, true, true>(i, gravity, strong, linlog, adjust, pos, mass, size, off, inc,
                                   fa);
}

// ---- 7. swinging, traction, FP64 totals and the speed update --------------
// Per node: swing in the device precision (kept for the displacement); the
// totals over the nodes that can move are summed in double: per thread over a
// fixed set of nodes, per block in a fixed tree order, then by the last block
// over the block partials with Neumaier compensation. The same block then
// updates Gephi's adaptive speed in double (reference
// src/forceatlas2.c:443-485), so no total ever goes to the host.

__device__ __forceinline__ void neumaier(double &s, double &c, double v)
{
    const double t = __dadd_rn(s, v);
    if (fabs(s) >= fabs(v))
        c = __dadd_rn(c, __dadd_rn(__dsub_rn(s, t), v));
    else
        c = __dadd_rn(c, __dadd_rn(__dsub_rn(v, t), s));
    s = t;
}

__device__ inline void update_speed_dev(SpeedState *st, double tsw, double ttr)
{
    double speed = st->speed, eff = st->efficiency;
    st->total_swinging = tsw;
    st->total_traction = ttr;
    if (!(tsw > 0)) return;
    const int n = st->n;
    const double jitter = st->jitter_tolerance;
    const double est = __dmul_rn(0.05, sqrt((double) n));
    const double min_jt = sqrt(est), max_jt = 10.0;
    double jt = __ddiv_rn(__dmul_rn(est, ttr), __dmul_rn((double) n, (double) n));
    if (jt > max_jt) jt = max_jt;
    if (jt < min_jt) jt = min_jt;
    jt = __dmul_rn(jt, jitter);
    if (tsw > __dmul_rn(2.0, ttr)) {
        if (eff > 0.05) eff = __dmul_rn(eff, 0.5);
        if (jt < jitter) jt = jitter;
    }
    const double target = __ddiv_rn(__dmul_rn(__dmul_rn(jt, eff), ttr), tsw);
    if (tsw > __dmul_rn(jt, ttr)) {
        if (eff > 0.05) eff = __dmul_rn(eff, 0.7);
    } else if (speed < 1000) {
        eff = __dmul_rn(eff, 1.3);
    }
    const double rise = __dsub_rn(target, speed);
    const double cap = __dmul_rn(0.5, speed);
    speed = __dadd_rn(speed, rise < cap ? rise : cap);
    st->speed = speed;
    st->efficiency = eff;
}

// In the FP64 path, up to this many nodes the totals are summed serially in
// node order, the reference's order (src/forceatlas2.c:770-775): the speed,
// hence the whole trajectory, is then the reference's bit for bit. Beyond,
// and always in the FP32 path (whose forces differ from the reference's in
// any case), a fixed-order tree: float-float in FP32, with compensation in
// FP64. A serial chain of double additions costs about 70 ns an addition
// on a GB300 (0.28 ms an iteration at 2000 nodes).
constexpr int SERIAL_TOTALS_MAX = 2048;
template <class R> __host__ __device__ constexpr bool serial_totals(int n)
{
    return sizeof(R) == 8 && n <= SERIAL_TOTALS_MAX;
}

// Per-thread sums of swinging and traction over the nodes that can move:
// float-float in the FP32 path, double in the FP64 path.
template <class R> struct SwingAcc {
    ff2 s = ff2{0.0f, 0.0f}, t = ff2{0.0f, 0.0f};
    double ds = 0.0, dt = 0.0;
};

// Node i's swinging (kept for the displacement) and traction
// (reference src/forceatlas2.c:758-775), added to the thread's sums.
template <class R>
__device__ __forceinline__ void swing_node(int i, int n, const typename RT<R>::R2 *f,
                                           const typename RT<R>::R2 *fold, const R *mass,
                                           const uint8_t *fixed, R *sw, R *tr, SwingAcc<R> &acc);

// The same from the node's force a, its previous force b and mass m, loaded
// by the caller.
template <class R>
__device__ __forceinline__ void swing_node_v(int i, typename RT<R>::R2 a, typename RT<R>::R2 b,
                                             R m, const uint8_t *fixed, R *sw, R *tr,
                                             SwingAcc<R> &acc)
{
    const R sx = b.x - a.x, sy = b.y - a.y;
    const R tx = b.x + a.x, ty = b.y + a.y;
    const R s = m * fsqrt(sx * sx + sy * sy);
    const R t = R(0.5) * m * fsqrt(tx * tx + ty * ty);
    sw[i] = s;
    if (tr) tr[i] = t; // kept for the serial totals, or on request
    if (fixed && fixed[i]) return;
    if constexpr (sizeof(R) == 4) {
        acc.s = ff_add(acc.s, ff_from((float) s));
        acc.t = ff_add(acc.t, ff_from((float) t));
    } else {
        acc.ds = __dadd_rn(acc.ds, (double) s);
        acc.dt = __dadd_rn(acc.dt, (double) t);
    }
}

template <class R>
__device__ __forceinline__ void swing_node(int i, int n, const typename RT<R>::R2 *f,
                                           const typename RT<R>::R2 *fold, const R *mass,
                                           const uint8_t *fixed, R *sw, R *tr, SwingAcc<R> &acc)
{
    const typename RT<R>::R2 a = f[i], b = fold[i];
    const R sx = b.x - a.x, sy = b.y - a.y;
    const R tx = b.x + a.x, ty = b.y + a.y;
    const R m = mass[i];
    const R s = m * fsqrt(sx * sx + sy * sy);
    const R t = R(0.5) * m * fsqrt(tx * tx + ty * ty);
    sw[i] = s;
    if (tr) tr[i] = t; // kept for the serial totals, or on request
    if (fixed && fixed[i]) return;
    if constexpr (sizeof(R) == 4) {
        acc.s = ff_add(acc.s, ff_from((float) s));
        acc.t = ff_add(acc.t, ff_from((float) t));
    } else {
        acc.ds = __dadd_rn(acc.ds, (double) s);
        acc.dt = __dadd_rn(acc.dt, (double) t);
    }
}

__device__ __forceinline__ ff2 ff_shfl_down(ff2 a, int o)
{
    return ff2{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
}

// The end of the totals, by every thread of every block of the kernel. Each
// block sums its nodes' values in a fixed tree order -- float-float in the
// FP32 path (FP32 operations only: a dependent FP64 add costs ~64 cycles on
// a GB300, and an SM's FP64 pipe completes 2 lanes a cycle), double in the
// FP64 path -- into a partial (a float-float pair (hi, lo) is the exact
// double hi + lo). The last block to finish sums the partials in a fixed
// order: in the FP64 path with Neumaier compensation in double; in the FP32
// path in float-float, then the warps' sums in double with Neumaier
// compensation -- or, up to SERIAL_TOTALS_MAX nodes in the FP64 path, the
// nodes serially in node order (the reference's order) -- and updates
// Gephi's adaptive speed in double.
template <class R>
__device__ __forceinline__ void swing_finish(SwingAcc<R> acc, int n, const uint8_t *fixed,
                                             const R *sw, const R *tr, double2 *partial,
                                             unsigned *ticket, SpeedState *st, int *status)
{
    __shared__ double ss[32], st_[32];
    __shared__ ff2 fss[32], fst[32];
    __shared__ int last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if constexpr (sizeof(R) == 4) {
        for (int o = 16; o > 0; o >>= 1) {
            acc.s = ff_add(acc.s, ff_shfl_down(acc.s, o));
            acc.t = ff_add(acc.t, ff_shfl_down(acc.t, o));
        }
        if (lane == 0) {
            fss[w] = acc.s;
            fst[w] = acc.t;
        }
    } else {
        acc.ds = warp_sum(acc.ds);
        acc.dt = warp_sum(acc.dt);
        if (lane == 0) {
            ss[w] = acc.ds;
            st_[w] = acc.dt;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if constexpr (sizeof(R) == 4) {
            ff2 a = fss[0], b = fst[0];
            for (int k = 1; k < nw; k++) {
                a = ff_add(a, fss[k]);
                b = ff_add(b, fst[k]);
            }
            // (hi, lo) of both sums: the exact doubles a.hi + a.lo, b.hi + b.lo
            reinterpret_cast<float4 *>(partial)[blockIdx.x] = make_float4(a.hi, a.lo, b.hi, b.lo);
        } else {
            double a = 0.0, b = 0.0, ca = 0.0, cb = 0.0;
            for (int k = 0; k < nw; k++) {
                neumaier(a, ca, ss[k]);
                neumaier(b, cb, st_[k]);
            }
            partial[blockIdx.x] = make_double2(__dadd_rn(a, ca), __dadd_rn(b, cb));
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double tsw = 0.0, ttr = 0.0;
    if (serial_totals<R>(n)) {
        // the block stages the nodes' values in shared memory (dynamic, 2n
        // reals; a fixed node's as +0, which leaves a sum unchanged), then
        // one thread adds them in node order: the chain waits on the adds
        // only, not on a load per node
        extern __shared__ __align__(16) unsigned char serial_smem[];
        R *ssw = reinterpret_cast<R *>(serial_smem), *str = ssw + n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const bool skip = fixed && fixed[i];
            ssw[i] = skip ? R(0) : __ldcg(sw + i);
            str[i] = skip ? R(0) : __ldcg(tr + i);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll 8
            for (int i = 0; i < n; i++) {
                tsw = __dadd_rn(tsw, (double) ssw[i]);
                ttr = __dadd_rn(ttr, (double) str[i]);
            }
        }
    } else if constexpr (sizeof(R) == 4) {
        // the partials per thread (strided, fixed order) and per warp in
        // float-float, whose same-sign sums lose about 2^-47 relative a step
        // (FP32 instructions: this block runs on one SM, whose FP64 pipe
        // completes 2 lanes a cycle); then the warps' sums in FP64 with
        // Neumaier compensation
        ff2 a = ff2{0.0f, 0.0f}, b = ff2{0.0f, 0.0f};
        const float4 *pf = reinterpret_cast<const float4 *>(partial);
        for (int k = threadIdx.x; k < (int) gridDim.x; k += blockDim.x) {
            const float4 v = __ldcg(pf + k);
            a = ff_add(a, ff2{v.x, v.y});
            b = ff_add(b, ff2{v.z, v.w});
        }
        for (int o = 16; o > 0; o >>= 1) {
            a = ff_add(a, ff_shfl_down(a, o));
            b = ff_add(b, ff_shfl_down(b, o));
        }
        __syncthreads();
        if (lane == 0) { // hi + lo is exact in double
            ss[w] = ff_to_double(a);
            st_[w] = ff_to_double(b);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t1 = 0.0, k1 = 0.0, t2 = 0.0, k2 = 0.0;
            for (int k = 0; k < nw; k++) {
                neumaier(t1, k1, ss[k]);
                neumaier(t2, k2, st_[k]);
            }
            tsw = __dadd_rn(t1, k1);
            ttr = __dadd_rn(t2, k2);
        }
    } else {
        double s1 = 0.0, c1 = 0.0, s2 = 0.0, c2 = 0.0;
        for (int k = threadIdx.x; k < (int) gridDim.x; k += blockDim.x) {
            const double2 v = __ldcg(partial + k);
            neumaier(s1, c1, v.x);
            neumaier(s2, c2, v.y);
        }
        double v1 = warp_sum(__dadd_rn(s1, c1)), v2 = warp_sum(__dadd_rn(s2, c2));
        __syncthreads();
        if (lane == 0) {
            ss[w] = v1;
            st_[w] = v2;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t1 = 0.0, k1 = 0.0, t2 = 0.0, k2 = 0.0;
            for (int k = 0; k < nw; k++) {
                neumaier(t1, k1, ss[k]);
                neumaier(t2, k2, st_[k]);
            }
            tsw = __dadd_rn(t1, k1);
            ttr = __dadd_rn(t2, k2);
        }
    }
    if (threadIdx.x == 0) {
        *ticket = 0u;
        if (!(tsw == tsw) || !(ttr == ttr)) {
            atomicOr(status + ST_ERROR, ERR_NAN);
            st->total_swinging = tsw;
            st->total_traction = ttr;
        } else {
            update_speed_dev(st, tsw, ttr);
        }
    }
}

// Attraction and gravity, then (the node's force complete) its swinging and
// traction, and the totals with the speed update: one thread per node, one
// launch for the attraction and the totals.
template <class R>
__global__ void __launch_bounds__(256)
k_attract_swing(int n, R gravity, int strong, int linlog, int adjust,
                const typename RT<R>::R2 *__restrict__ pos, const R *__restrict__ mass,
                const R *__restrict__ size, const int *__restrict__ off,
                const Inc<R> *__restrict__ inc, typename RT<R>::R2 *__restrict__ f,
                const typename RT<R>::R2 *__restrict__ fold, const uint8_t *__restrict__ fixed,
                R *__restrict__ sw, R *__restrict__ tr, double2 *__restrict__ partial,
                unsigned *__restrict__ ticket, SpeedState *__restrict__ st,
                int *__restrict__ status)
{
    SwingAcc<R> acc;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        attract_one<R, sizeof(R) == 4>(i, gravity, strong, linlog, adjust, pos, mass, size, off,
                                       inc, f);
        swing_node<R>(i, n, f, fold, mass, fixed, sw, tr, acc);
    }
    swing_finish<R>(acc, n, fixed, sw, tr, partial, ticket, st, status);
}

// The join of the attraction run beside the walk: a node's force is its
// repulsion (f) plus its gravity and attraction (fa), then its swinging and
// traction, and the totals with the speed update. Grid-stride over a few
// blocks per SM: few block partials for the last block to add up.
template <class R>
__global__ void __launch_bounds__(256)
k_join_swing(int n, const typename RT<R>::R2 *__restrict__ fa, typename RT<R>::R2 *__restrict__ f,
             const typename RT<R>::R2 *__restrict__ fold, const R *__restrict__ mass,
             const uint8_t *__restrict__ fixed, R *__restrict__ sw, R *__restrict__ tr,
             double2 *__restrict__ partial, unsigned *__restrict__ ticket,
             SpeedState *__restrict__ st, int *__restrict__ status)
{
    typedef typename RT<R>::R2 R2;
    SwingAcc<R> acc;
    // U nodes a round, their loads issued together; the nodes of a thread
    // are added to its sums in node order
    constexpr int U = 4;
    const int stride = gridDim.x * blockDim.x;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
        R2 r[U], a[U], b[U];
        R m[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * stride;
            if (i < n) {
                r[u] = f[i];
                a[u] = fa[i];
                b[u] = fold[i];
                m[u] = mass[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * stride;
            if (i >= n) break;
            const R2 t = mk2<R>(r[u].x + a[u].x, r[u].y + a[u].y);
            f[i] = t;
            swing_node_v<R>(i, t, b[u], m[u], fixed, sw, tr, acc);
        }
    }
    swing_finish<R>(acc, n, fixed, sw, tr, partial, ticket, st, status);
}

// f += fa (the forces of one evaluation, fa2cu_layout_forces, in the order
// the iteration adds them).
template <class R>
__global__ void __launch_bounds__(256)
k_add_forces(int n, const typename RT<R>::R2 *__restrict__ fa, typename RT<R>::R2 *__restrict__ f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const typename RT<R>::R2 r = f[i], a = fa[i];
    f[i] = mk2<R>(r.x + a.x, r.y + a.y);
}

// ---- 8. displacement (pipeline.cl:476-506) ---------------------------------

// The displacement (reference src/forceatlas2.c:780-802), fused with the
// bounding box of the new positions that the next iteration's Morton codes
// need: a grid-stride pass (the bounding box's block count) that moves every
// node that may move and folds every node's position into the block's
// minima / maxima, then bbox_finish (skipped when partial is null: exact
// layouts need no box). Once the layout has stopped on an error, positions
// are kept (the box is still computed).
template <class R>
__global__ void __launch_bounds__(256)
k_apply(int n, int adjust, const typename RT<R>::R2 *__restrict__ f,
        typename RT<R>::R2 *__restrict__ fold, const R *__restrict__ sw,
        const uint8_t *__restrict__ fixed, typename RT<R>::R2 *__restrict__ pos,
        const SpeedState *__restrict__ st, const int *__restrict__ status,
        R *__restrict__ partial, R *__restrict__ bbox, double *__restrict__ quant,
        unsigned *__restrict__ ticket)
{
    pdl_wait();
    const bool stopped = status[ST_ERROR] != 0;
    const R speed = (R) st->speed;
    R mnx = (R) INFINITY, mny = (R) INFINITY, mxx = -(R) INFINITY, mxy = -(R) INFINITY;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        typename RT<R>::R2 p = pos[i];
        if (!stopped) {
            const typename RT<R>::R2 a = f[i];
            fold[i] = a;
            if (!(fixed && fixed[i])) {
                R factor;
                if (adjust) {
                    const R df = fsqrt(a.x * a.x + a.y * a.y);
                    factor = fdiv(R(0.1) * speed, R(1) + fsqrt(speed * sw[i]));
                    if (df > R(0)) {
                        if (factor * df > R(10)) factor = fdiv(R(10), df);
                    } else {
                        factor = R(0);
                    }
                } else {
                    factor = fdiv(speed, R(1) + fsqrt(speed * sw[i]));
                }
                p.x += a.x * factor;
                p.y += a.y * factor;
                pos[i] = p;
            }
        }
        mnx = cl_min(mnx, p.x);
        mny = cl_min(mny, p.y);
        mxx = cl_max(mxx, p.x);
        mxy = cl_max(mxy, p.y);
    }
    if (partial) // (uniform: a layout without a tree has no box to keep)
        bbox_finish<R>(mnx, mny, mxx, mxy, partial, bbox, quant, ticket);
}

// ---- conversions between the host's doubles and the device layout --------

template <class R>
__global__ void __launch_bounds__(256)
k_pos_in(int n, const double *__restrict__ xy, typename RT<R>::R2 *__restrict__ pos)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[i] = mk2<R>((R) xy[i], (R) xy[n + i]);
}

template <class R>
__global__ void __launch_bounds__(256)
k_pos_out(int n, const typename RT<R>::R2 *__restrict__ pos, double *__restrict__ xy)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const typename RT<R>::R2 p = pos[i];
    xy[i] = (double) p.x;
    xy[n + i] = (double) p.y;
}

template <class R>
__global__ void __launch_bounds__(256)
k_real_in(int n, const double *__restrict__ in, R *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (R) in[i];
}

template <class R>
__global__ void __launch_bounds__(256)
k_inc_in(int ninc, const int *__restrict__ node, const double *__restrict__ coef,
         Inc<R> *__restrict__ inc)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ninc) return;
    Inc<R> c;
    c.j = node[e];
    c.coef = (R) coef[e];
    inc[e] = c;
}

// (x, y, m, r) records of every node in original order (the exact kernel's
// input); r = 0 unless adjust.
template <class R>
__global__ void __launch_bounds__(256)
k_pack(int n, int adjust, const typename RT<R>::R2 *__restrict__ pos,
       const R *__restrict__ mass, const R *__restrict__ size,
       typename RT<R>::R4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const typename RT<R>::R2 p = pos[i];
    out[i] = mk4<R>(p.x, p.y, mass[i], adjust ? size[i] : R(0));
}

// Same records from four host-layout double arrays (fa2_gpu_repulse_*).
template <class R>
__global__ void __launch_bounds__(256)
k_pack_host(int n, const double *__restrict__ x, const double *__restrict__ y,
            const double *__restrict__ m, const double *__restrict__ s,
            typename RT<R>::R4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = mk4<R>((R) x[i], (R) y[i], (R) m[i], s ? (R) s[i] : R(0));
}

// Forces to two double arrays, through a permutation when perm != NULL
// (reference src/gpu.c:520-533).
template <class R>
__global__ void __launch_bounds__(256)
k_forces_out(int n, const typename RT<R>::R2 *__restrict__ f, const int *__restrict__ perm,
             double *__restrict__ fx, double *__restrict__ fy)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = perm ? perm[k] : k;
    const typename RT<R>::R2 v = f[k];
    fx[i] = (double) v.x;
    fy[i] = (double) v.y;
}

// ---- exact repulsion: the n-body tile kernel ------------------------------
// Each thread owns IPT nodes (i, i + T, ...) and sums over every j in
// ascending order, as the reference (src/forceatlas2.c:278-294). Tiles of
// (x, y, m, r) records are staged in shared memory by TMA bulk copies
// (cp.async.bulk, completion on an mbarrier), two tiles in flight. The pair
// i == j contributes exactly zero (xd = yd = 0 with a finite factor), so no
// test is needed. Every mbarrier wait is bounded in time: on expiry the
// kernel records ERR_WAIT, drains its copies in flight and returns.

#define FA2_EXACT_THREADS 256
#ifndef FA2_EXACT_IPT_F32
#define FA2_EXACT_IPT_F32 4 // nodes per thread in FP32 (FP64: 1)
#endif

// Records per tile of the all-pairs kernel (8 KB of records, double-buffered).
template <class R> __host__ __device__ constexpr int exact_tile()
{
    return 8192 / (int) sizeof(typename RT<R>::R4);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t) __cvta_generic_to_shared(p);
}


__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes,
                                            uint64_t *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, unsigned phase)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(phase)
                 : "memory");
    return ok != 0;
}

// Wait for a phase of `bar`, for at most `limit_ns` nanoseconds.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned phase,
                                          unsigned long long limit_ns)
{
    if (mbar_try(bar, phase)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try(bar, phase)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Block (x, y) sums, for its FA2_EXACT_THREADS * IPT nodes, the sources
// [y seg, min(n, (y + 1) seg)) (seg a multiple of the tile): into f when the
// grid has one row (every j, ascending: the reference's order), else into
// row y of `partial` (n entries per row), summed by k_exact_sum.
template <class R, bool ADJUST, int IPT>
__global__ void __launch_bounds__(FA2_EXACT_THREADS)
k_exact(int n, R scaling, const typename RT<R>::R4 *__restrict__ nodes,
        typename RT<R>::R2 *__restrict__ f, typename RT<R>::R2 *__restrict__ partial, int seg,
        int *__restrict__ status)
{
    typedef typename RT<R>::R4 R4;
    constexpr int TILE = exact_tile<R>();
    extern __shared__ __align__(128) unsigned char smem[];
    R4 *tile = reinterpret_cast<R4 *>(smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * TILE * sizeof(R4));
    __shared__ int failed;

    R xi[IPT], yi[IPT], mi[IPT], si[IPT], smi[IPT], ax[IPT], ay[IPT];
    const int i0 = blockIdx.x * (FA2_EXACT_THREADS * IPT) + threadIdx.x;
#pragma unroll
    for (int u = 0; u < IPT; u++) {
        const int i = i0 + u * FA2_EXACT_THREADS;
        const R4 p = nodes[i < n ? i : n - 1];
        xi[u] = p.x;
        yi[u] = p.y;
        mi[u] = p.z;
        si[u] = p.w;
        smi[u] = scaling * p.z;
        ax[u] = ay[u] = R(0);
    }
    const int j0 = blockIdx.y * seg, j1 = min(n, j0 + seg);
    const R4 *src = nodes + j0;
    const int ntiles = (j1 - j0 + TILE - 1) / TILE;
    if (threadIdx.x == 0) {
        failed = 0;
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 0; t < 2 && t < ntiles; t++) {
            const int cnt = min(TILE, j1 - j0 - t * TILE);
            tma_load_1d(tile + t * TILE, src + (size_t) t * TILE, cnt * (unsigned) sizeof(R4),
                        &bar[t]);
        }
    }
    for (int t = 0; t < ntiles; t++) {
        const int b = t & 1;
        if (!mbar_wait(&bar[b], (t >> 1) & 1, 2000000000ull)) failed = 1;
        __syncthreads();
        if (failed) {
            // drain what may still be in flight, then give up
            if (threadIdx.x == 0) {
                atomicOr(status + ST_ERROR, ERR_WAIT);
                for (int u = t; u < t + 2 && u < ntiles; u++)
                    mbar_wait(&bar[u & 1], (u >> 1) & 1, 2000000000ull);
            }
            __syncthreads();
            return;
        }
        const R4 *q = tile + b * TILE;
        const int cnt = min(TILE, j1 - j0 - t * TILE);
        if constexpr (sizeof(R) == 4 && !ADJUST) {
            // FP32: 7 FP32-pipe operations and one MUFU reciprocal per
            // pair; the thread's scaling * m_i multiplies the sums once at
            // the end. d2 carries 1e-30 (d2 = xd^2 + (yd^2 + 1e-30), one FMA
            // each): a coincident pair (xd = yd = 0) then has a finite
            // factor below 1e30 * m_j, so its term is 0 -- the reference's
            // factor for d2 = 0 -- without a compare; any other pair of
            // float positions is at least ~1e-14 apart in d2 for
            // coordinates of 1e-3 or more, which the 1e-30 leaves unchanged
            // to float precision.
#pragma unroll 4
            for (int jj = 0; jj < cnt; jj++) {
                const R4 p = q[jj];
#pragma unroll
                for (int u = 0; u < IPT; u++) {
                    const float xd = xi[u] - p.x, yd = yi[u] - p.y;
                    const float d2 = fmaf(xd, xd, fmaf(yd, yd, 1e-30f));
                    const float g = p.z * __fdividef(1.0f, d2);
                    ax[u] = fmaf(xd, g, ax[u]);
                    ay[u] = fmaf(yd, g, ay[u]);
                }
            }
        } else {
#pragma unroll 4
            for (int jj = 0; jj < cnt; jj++) {
                const R4 p = q[jj];
#pragma unroll
                for (int u = 0; u < IPT; u++) {
                    const R xd = xi[u] - p.x, yd = yi[u] - p.y;
                    const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi[u] * p.z,
                                                      si[u] + p.w, scaling);
                    ax[u] += xd * g;
                    ay[u] += yd * g;
                }
            }
        }
        __syncthreads(); // every thread is done with buffer b
        if (threadIdx.x == 0 && t + 2 < ntiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const int cnt2 = min(TILE, j1 - j0 - (t + 2) * TILE);
            tma_load_1d(tile + b * TILE, src + (size_t) (t + 2) * TILE,
                        cnt2 * (unsigned) sizeof(R4), &bar[b]);
        }
    }
#pragma unroll
    for (int u = 0; u < IPT; u++) {
        const int i = i0 + u * FA2_EXACT_THREADS;
        if (sizeof(R) == 4 && !ADJUST) {
            ax[u] *= smi[u];
            ay[u] *= smi[u];
        }
        if (i < n) {
            if (partial)
                partial[(size_t) blockIdx.y * n + i] = mk2<R>(ax[u], ay[u]);
            else
                f[i] = mk2<R>(ax[u], ay[u]);
        }
    }
}

// The rows of k_exact's partial sums, in row order.
template <class R>
__global__ void __launch_bounds__(256)
k_exact_sum(int n, int rows, const typename RT<R>::R2 *__restrict__ partial,
            typename RT<R>::R2 *__restrict__ f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    typename RT<R>::R2 a = partial[i];
    for (int r = 1; r < rows; r++) {
        const typename RT<R>::R2 b = partial[(size_t) r * n + i];
        a.x += b.x;
        a.y += b.y;
    }
    f[i] = a;
}

template <class R> constexpr size_t exact_smem_bytes()
{
    return 2 * (size_t) exact_tile<R>() * sizeof(typename RT<R>::R4) + 2 * sizeof(uint64_t);
}

// Rows of source ranges for an n-node all-pairs sum on a GPU of `sms` SMs:
// enough blocks for about six per SM, each range at least two tiles long;
// 1 in double (every node sums every j in order) or when n alone fills the
// GPU.
template <class R> int exact_rows(int n, int sms, int ipt)
{
    if (sizeof(R) != 4) return 1;
    const int nb = (n + FA2_EXACT_THREADS * ipt - 1) / (FA2_EXACT_THREADS * ipt);
    const int want = (6 * sms + nb - 1) / nb;
    const int most = n / (2 * exact_tile<R>());
    int rows = want < most ? want : most;
    if (rows > 16) rows = 16;
    return rows < 1 ? 1 : rows;
}


// ---- quadtree traversal of fa2_gpu_repulse_bh (reference src/gpu.c:78-123)
// Regions of the host's Gephi quadtree, converted on the device.

template <class R>
__global__ void __launch_bounds__(256)
k_qregions(int nreg, const fa2_region *__restrict__ reg, QRegion<R> *__restrict__ out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nreg) return;
    const fa2_region g = reg[r];
    QRegion<R> q;
    q.rr = mk4<R>((R) g.cx, (R) g.cy, (R) g.mass, (R) (g.size * g.size));
    q.ri = make_int4(g.start, g.count, g.nchild > 0 ? g.child + g.nchild - 1 : -1, g.skip);
    out[r] = q;
}

// Stackless walk over the quadtree: go down to the last child or jump to
// `skip` (the previous sibling, else the parent's skip), the visiting order of
// the CPU's stack (src/forceatlas2.c:326-368). Nodes in tree order; the
// output is in tree order too.
template <class R, bool ADJUST>
__global__ void __launch_bounds__(256)
k_qtraverse(int n, R scaling, R theta2, double theta2d, const typename RT<R>::R4 *__restrict__ p,
            const double *__restrict__ px, const double *__restrict__ py,
            const QRegion<R> *__restrict__ reg, const fa2_region *__restrict__ raw, int nreg,
            typename RT<R>::R2 *__restrict__ f, int *__restrict__ status)
{
    typedef typename RT<R>::R4 R4;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const R4 me = p[k];
    const R xi = me.x, yi = me.y, mi = me.z, si = me.w;
    R ax = R(0), ay = R(0);
    int cur = 0, j = 0, jend = -1;
    const int cap = 2 * nreg + 2 * n + 64;
    for (int step = 0;; step++) {
        if (step > cap || cur >= nreg || jend >= n) {
            atomicOr(status + ST_ERROR, ERR_BOUNDS);
            break;
        }
        if (j <= jend) {
            if (j != k) {
                const R4 q = p[j];
                const R xd = xi - q.x, yd = yi - q.y;
                const R g = rep_factor<R, ADJUST>(xd * xd + yd * yd, mi * q.z,
                                                  si + q.w, scaling);
                ax += xd * g;
                ay += yd * g;
            }
            ++j;
            continue;
        }
        if (cur < 0) break;
        const QRegion<R> q = reg[cur];
        if (q.ri.y > 1) {
            const R xd = xi - q.rr.x, yd = yi - q.rr.y;
            const R d2 = xd * xd + yd * yd;
            const R lhs = d2 * theta2;
            bool far = lhs > q.rr.w;
            if (sizeof(R) == 4 && fabs_r(lhs - q.rr.w) <= R(DECIDE_BAND) * q.rr.w) {
                // the host's double region and node, as the CPU decides
                const double ex = __dsub_rn(px[k], raw[cur].cx), ey = __dsub_rn(py[k], raw[cur].cy);
                const double sz = raw[cur].size;
                far = __dmul_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), theta2d) >
                      __dmul_rn(sz, sz);
            }
            if (far) {
                const R g = fdiv(scaling * (mi * q.rr.z), d2);
                ax += xd * g;
                ay += yd * g;
                cur = q.ri.w;
                continue;
            }
            if (q.ri.z >= 0) {
                cur = q.ri.z;
                continue;
            }
        }
        j = q.ri.x;
        jend = q.ri.x + q.ri.y - 1;
        cur = q.ri.w;
    }
    f[k] = mk2<R>(ax, ay);
}

} // namespace fa2cu
