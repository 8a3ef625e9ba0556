// Barnes-Hut traversal, form "fast": FP64-accurate results from float-float
// arithmetic on the FP32 pipe.
//
// On GB300 the FP64 pipe runs at about 1/70 of the FP32 pipe, and f32<->f64
// conversions at the FP64 rate, so the FP64 pair loop of k_traverse_exact is
// bound at ~1 TFLOP/s.  This kernel keeps every pair term to ~2^-44 relative
// (the sum of ~5e4 such terms is far inside the 1e-10 relative-L2 contract)
// while issuing only FP32 instructions in the hot loop:
//
//  * Coordinates are shifted to the tree's box centre and scaled by a power
//    of two into [-1/2, 1/2]; each coordinate is stored as hi + lo with hi on
//    the 2^-23 grid and lo on the 2^-47 grid (|lo| <= 2^-24), so hi_j - hi_i
//    and lo_j - lo_i are exact in FP32 and the displacement is exact up to
//    the 2^-48 representation of the coordinates.  Masses are scaled by a power
//    of two into [-1, 1] and split hi + lo.  Scales are undone in FP64.
//  * r^2 + eps^2 is summed error-free (two-product squares, TwoSum of the
//    high parts); (r^2)^(-3/2) is the hardware rsqrt refined by one
//    correction step, w = y^3 (1 + 3e/2 + 15e^2/8) with e = 1 - r^2 y^2
//    computed exactly (Newton-Raphson for the inverse square root, carried
//    to second order; the softened term pair_ff_soft stops at first order);
//    m * w * dx and the accumulation are float-float (Dekker/Knuth
//    two-product and TwoSum).
//  * A pair's relative error is dominated by the 2^-48 coordinate
//    representation: about 2^-48 / sqrt(r^2 + eps^2).  With a softening
//    that bounds r^2 + eps^2 from below ((eps s)^2 >= 2^-33) every pair is
//    float-float and the range test is compiled out; otherwise pairs with
//    r^2 + eps^2 below 2^-26 in normalised units (softened distance under
//    2^-13 of the box half-size), or outside the FP32 range, are evaluated
//    in FP64 from the FP64 arrays, so a float-float pair stays below 2^-35.
//  * The opening decision is the reference's, bit for bit: a FP32 test
//    decides every node whose ratio is clearly above or below theta, and
//    nodes inside a small error band are decided by the exact FP64 test of
//    k_traverse_exact (bh.py:576-601).  Every lane therefore evaluates
//    exactly the reference's interaction set for its target.
#include "fast.cuh"

namespace bhut {

constexpr int kFastWarps = 4;
constexpr int kFastThreads = kFastWarps * kWarp;
// Tuning (overridable at build time): resident blocks per SM for the fast
// form (6: 24 warps per SM, registers capped at 80) and the unroll factors
// of the leaf pair loops.  Swept on GB300 at 1M Plummer: unroll 4 / 8 beat
// 1-2 / 1-4 by 2-10 %; 5 blocks per SM (96 registers) gains nothing.
#ifndef BHUT_FAST_BLOCKS
#define BHUT_FAST_BLOCKS 6
#endif
#ifndef BHUT_F32_UNROLL
#define BHUT_F32_UNROLL 8
#endif
// Self accelerations of few targets: up to this many lanes per target (1, 2
// or 4; k_traverse_fast_lpt).
#ifndef BHUT_FAST_MAX_LPT
#define BHUT_FAST_MAX_LPT 4
#endif
// ... chosen so that at least this many warps per SM share the work
#ifndef BHUT_FAST_LPT_WARPS_PER_SM
#define BHUT_FAST_LPT_WARPS_PER_SM 8
#endif
static_assert(BHUT_FAST_MAX_LPT == 1 || BHUT_FAST_MAX_LPT == 2 || BHUT_FAST_MAX_LPT == 4 ||
              BHUT_FAST_MAX_LPT == 8, "lanes per target: 1, 2, 4 or 8");
// Checked path (small or no softening): split sparse leaf visits (1) or not.
#ifndef BHUT_CHECK_SPLIT
#define BHUT_CHECK_SPLIT 1
#endif
constexpr int kFastBlocksPerSM = BHUT_FAST_BLOCKS;
constexpr int kF32Unroll = BHUT_F32_UNROLL;

// ---------------------------------------------------------------------------
// frame (normalisation) derived from the tree's bounding box
// ---------------------------------------------------------------------------
__global__ void k_frame(const double* __restrict__ box, int dim, FastFrame* __restrict__ f)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        frame_from_box(box, dim, f);
        frame_unit_mass(box[6], box[15] != 0.0, f);
    }
}

__global__ void k_ff_particles(const double* __restrict__ sx, const double* __restrict__ sy,
                               const double* __restrict__ sz, const double* __restrict__ sm,
                               int64_t n, int dim, const FastFrame* __restrict__ fr,
                               float4* __restrict__ ph, float4* __restrict__ pl)
{
    const FastFrame f = *fr;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 h, l;
        split_grid(__dmul_rn(__dsub_rn(sx[i], f.c[0]), f.s), h.x, l.x);
        split_grid(__dmul_rn(__dsub_rn(sy[i], f.c[1]), f.s), h.y, l.y);
        if (dim == 3) split_grid(__dmul_rn(__dsub_rn(sz[i], f.c[2]), f.s), h.z, l.z);
        else h.z = l.z = 0.0f;
        if (f.unit) { h.w = 1.0f; l.w = 0.0f; }   // every mass is m0: exactly 1 in units of m0
        else split_plain(__dmul_rn(sm[i], f.ms), h.w, l.w);
        ph[i] = h;
        pl[i] = l;
    }
}

__global__ void k_ff_nodes(TreeDev t, const double* __restrict__ center,
                           const FastFrame* __restrict__ fr, float4* __restrict__ nh,
                           float4* __restrict__ nl, float* __restrict__ nsize,
                           float* __restrict__ ndelta, const double* __restrict__ quad,
                           float4* __restrict__ nq0, float2* __restrict__ nq1,
                           int4* __restrict__ nhdr)
{
    const FastFrame f = *fr;
    const int dim = t.dim;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < t.m;
         k += (int64_t)gridDim.x * blockDim.x) {
        NodeCM c = t.cm[k];

        float4 h, l;
        // a node's COM lies inside the box: |u| <= 1 up to rounding
        split_grid(__dmul_rn(__dsub_rn(c.x, f.c[0]), f.s), h.x, l.x);
        split_grid(__dmul_rn(__dsub_rn(c.y, f.c[1]), f.s), h.y, l.y);
        if (dim == 3) split_grid(__dmul_rn(__dsub_rn(c.z, f.c[2]), f.s), h.z, l.z);
        else h.z = l.z = 0.0f;
        split_plain(__dmul_rn(c.w, f.ms), h.w, l.w);
        nh[k] = h;
        nl[k] = l;
        nsize[k] = __double2float_rn(__dmul_rn(t.size[k], f.s));
        // distance between the centre of mass and the AABB centre (offset MAC)
        double dd = 0.0;
        for (int d = 0; d < dim; d++) {
            const double cc = d == 0 ? c.x : (d == 1 ? c.y : c.z);
            const double v = cc - center[k * dim + d];
            dd += v * v;
        }
        ndelta[k] = __double2float_ru(sqrt(dd) * f.s);
        // header: leaf (-1, start, count, mass != 0); internal (first child,
        // size, |com - centre| as float bits, mass != 0)
        const int fc = t.first_child[k];
        nhdr[k] = fc < 0 ? make_int4(fc, t.start[k], t.count[k], c.w != 0.0)
                         : make_int4(fc, __float_as_int(nsize[k]), __float_as_int(ndelta[k]),
                                     c.w != 0.0);
        if (quad) {   // mass x length^2: scale by ms s^2
            const double qs = f.ms * f.s * f.s;
            const double* q = quad + 6 * k;
            nq0[k] = make_float4((float)(q[0] * qs), (float)(q[1] * qs), (float)(q[2] * qs),
                                 (float)(q[3] * qs));
            nq1[k] = make_float2((float)(q[4] * qs), (float)(q[5] * qs));
        }
    }
}

// Targets: grid split when inside the box (|u| <= 1), plain split otherwise;
// th.w = 1 marks a target outside the box, tl.w = max |u|.
__global__ void k_ff_targets(const double* __restrict__ tx, const double* __restrict__ ty,
                             const double* __restrict__ tz, int64_t nt, int dim,
                             const FastFrame* __restrict__ fr, float4* __restrict__ th,
                             float4* __restrict__ tl)
{
    const FastFrame f = *fr;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt;
         i += (int64_t)gridDim.x * blockDim.x) {
        double u[3] = {__dmul_rn(__dsub_rn(tx[i], f.c[0]), f.s),
                       __dmul_rn(__dsub_rn(ty[i], f.c[1]), f.s),
                       dim == 3 ? __dmul_rn(__dsub_rn(tz[i], f.c[2]), f.s) : 0.0};
        double amax = fmax(fabs(u[0]), fmax(fabs(u[1]), fabs(u[2])));
        bool inside = amax <= 1.0;
        float hh[3], ll[3];
        for (int d = 0; d < 3; d++) {
            if (inside) split_grid(u[d], hh[d], ll[d]);
            else split_plain(u[d], hh[d], ll[d]);
        }
        th[i] = make_float4(hh[0], hh[1], hh[2], inside ? 0.0f : 1.0f);
        tl[i] = make_float4(ll[0], ll[1], ll[2], __double2float_ru(amax));
    }
}

// ---------------------------------------------------------------------------
// the traversal
// ---------------------------------------------------------------------------
struct FastArgs {
    const float4* th;        // target hi (w: outside-box flag); NULL: the particles themselves
    const float4* tl;        // target lo (w: max |u|)
    const double* tx;        // target FP64 (fallbacks)
    const double* ty;
    const double* tz;
    const int32_t* self_id;
    const int32_t* out_idx;
    int64_t nt;
    double theta, eps, G;
    float e2h, e2l;          // (eps * s)^2 as float-float
    double* out;
    unsigned* err;
    unsigned long long* stats;
    int mac;                 // 0: reference criterion, 1: offset criterion (fp32 form)
};

// leaf_block_soft for the checked path (targets inside the box, softening
// too small to bound r^2 + eps^2 from below: pair_ff with the range test,
// pairs below kTinyRCheck taken in FP64 from the FP64 particle arrays).  The
// split is the same; a lane that works for another lane's target also
// takes that target's FP64 pairs (the target's FP64 coordinates come by
// shuffle) and the group adds its FP64 partial sums like the float-float
// ones.  `nfb` counts the FP64 pairs a lane evaluated.
template <int DIM>
__device__ __forceinline__ void leaf_block_check(unsigned mask, int lane, const float* Th,
                                                 const float* Tl, double x, double y, double z,
                                                 const float4* sh, const float4* sl, int cn,
                                                 int first, const TreeDev& t, float e2h,
                                                 float e2l, double eps2, float* ah, float* al,
                                                 double* a64, unsigned& nfb)
{
    const unsigned FULL = 0xffffffffu;
    const bool mine = (mask >> lane) & 1u;
    const int k = __popc(mask);
    if (k == 0) return;
    if (k > kSplitMaxK || !BHUT_CHECK_SPLIT) {
        if (mine) {
            unsigned fb = 0;
#pragma unroll (kFFUnroll)
            for (int q = 0; q < cn; q++)
                fb |= (unsigned)!pair_ff<DIM, false, true>(Th, Tl, sh[q], sl[q], e2h, e2l, ah,
                                                           al) << q;
            while (fb) {
                const int gi = first + __ffs(fb) - 1;
                fb &= fb - 1;
                pair_fp64<DIM>(x, y, z, t.sx[gi], t.sy[gi], DIM == 3 ? t.sz[gi] : 0.0, t.sm[gi],
                               eps2, a64);
                nfb++;
            }
        }
        return;
    }
    int f = 2;
    while (f * 2 * k <= kWarp) f *= 2;
    const int r = lane / f, sub = lane & (f - 1);
    const bool work = r < k;
    const int owner = nth_set_bit(mask, work ? r : 0);
    float T[3] = {0.f, 0.f, 0.f}, L[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        T[c] = __shfl_sync(FULL, Th[c], owner);
        L[c] = __shfl_sync(FULL, Tl[c], owner);
    }
    const double X = __shfl_sync(FULL, x, owner), Y = __shfl_sync(FULL, y, owner);
    const double Z = __shfl_sync(FULL, z, owner);
    float ph[3] = {0.f, 0.f, 0.f}, pl[3] = {0.f, 0.f, 0.f};
    double p64[3] = {0.0, 0.0, 0.0};
    if (work) {
        unsigned fb = 0;
#pragma unroll (kSplitUnroll)
        for (int q = sub; q < cn; q += f)
            fb |= (unsigned)!pair_ff<DIM, false, true>(T, L, sh[q], sl[q], e2h, e2l, ph, pl) << q;
        while (fb) {
            const int gi = first + __ffs(fb) - 1;
            fb &= fb - 1;
            pair_fp64<DIM>(X, Y, Z, t.sx[gi], t.sy[gi], DIM == 3 ? t.sz[gi] : 0.0, t.sm[gi],
                           eps2, p64);
            nfb++;
        }
    }
    for (int o = f >> 1; o >= 1; o >>= 1) {
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            const float bh = __shfl_down_sync(FULL, ph[c], o);
            const float bl = __shfl_down_sync(FULL, pl[c], o);
            ff_add(ph[c], pl[c], bh, bl);
            p64[c] = __dadd_rn(p64[c], __shfl_down_sync(FULL, p64[c], o));
        }
    }
    const int leader = mine ? __popc(mask & ((1u << lane) - 1u)) * f : 0;
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const float gh = __shfl_sync(FULL, ph[c], leader);
        const float gl = __shfl_sync(FULL, pl[c], leader);
        const double g64 = __shfl_sync(FULL, p64[c], leader);
        if (mine) {
            ff_add(ah[c], al[c], gh, gl);
            a64[c] = __dadd_rn(a64[c], g64);
        }
    }
}

// SOFT_PATH (= !FAR && !CHECK): every pair is taken by pair_ff_soft (no
// FP64 fallback); UNIT: leaf pairs skip the mass product (unit masses).
// LPT > 1 (soft path only): LPT consecutive lanes hold the same target; they
// take the same opening decisions, share its leaf pairs (lane j of the group
// takes pairs j, j + LPT, ...), the group's first lane alone adds monopoles
// and counts, and the caller adds the lanes' sums.
template <int DIM, bool FAR, bool CHECK, bool UNIT = false, int LPT = 1>
__device__ __forceinline__ void walk(const TreeDev& t, const FastTree& ft, const FastArgs& a,
                                     int w, int lane, bool valid, int64_t me_sorted, const float* Th,
                                     const float* Tl, float band_abs, double x, double y, double z,
                                     float* ah, float* al, double* a64, int2 (*stack)[kStackDepth],
                                     float4 (*sh)[kWarp], float4 (*sl)[kWarp],
                                     unsigned* cnt, bool& overflow)
{
    static_assert(LPT == 1 || (!FAR && !CHECK), "lane groups serve the soft path only");
    const unsigned FULL = 0xffffffffu;
    const float theta_f = (float)a.theta;
    const double eps2 = __dmul_rn(a.eps, a.eps);
    const bool lead = (lane & (LPT - 1)) == 0;   // first lane of the target's group
    const int sub = lane & (LPT - 1);
    const unsigned live = __ballot_sync(FULL, valid);
    if (lane == 0) stack[w][0] = make_int2(0, (int)live);
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int2 e = stack[w][--sp];
        __syncwarp();
        const int node = e.x;
        const unsigned mask = (unsigned)e.y;
        const bool act = (mask >> lane) & 1u;
        cnt[2] += act && lead;
        const int4 hd = ft.nhdr[node];   // (first_child, start, count, mass != 0)
        if (!hd.w) continue;              // mass == 0 skip (bh.py:514)
        const int fc = hd.x;
        if (fc < 0) {
            const int s = hd.y, c = hd.z;
            for (int b = 0; b < c; b += kWarp) {
                const int jj = b + lane;
                if (jj < c) {
                    sh[w][lane] = ft.ph[s + jj];
                    sl[w][lane] = ft.pl[s + jj];
                }
                __syncwarp();
                const int cn = min(kWarp, c - b);
                if (act && lead) {
                    // The target itself (self mode: sorted index `me_sorted`)
                    // sits at zero displacement and adds exactly zero, so it
                    // is not skipped; it is only left out of the pair count
                    // (bh.py:254).
                    cnt[0] += cn - (me_sorted >= s + b && me_sorted < s + b + cn);
                }
                if (!FAR && !CHECK && LPT == 1) {
                    leaf_block_soft<DIM, UNIT>(mask, lane, Th, Tl, sh[w], sl[w], cn, a.e2h, a.e2l,
                                               ah, al);
                } else if (!FAR && !CHECK) {
                    if (act) {
#pragma unroll (kSplitUnroll)
                        for (int q = sub; q < cn; q += LPT)
                            pair_ff_soft<DIM, UNIT>(Th, Tl, sh[w][q], sl[w][q], a.e2h, a.e2l, ah,
                                                    al);
                    }
                } else if (!FAR) {
                    leaf_block_check<DIM>(mask, lane, Th, Tl, x, y, z, sh[w], sl[w], cn, s + b, t,
                                          a.e2h, a.e2l, eps2, ah, al, a64, cnt[4]);
                } else if (act) {
                    unsigned fb = 0;   // pairs left to FP64 (rare), taken after the loop
#pragma unroll (kFFUnroll)
                    for (int q = 0; q < cn; q++)
                        fb |= (unsigned)!pair_ff<DIM, FAR, CHECK>(Th, Tl, sh[w][q], sl[w][q],
                                                                  a.e2h, a.e2l, ah, al) << q;
                    while (fb) {
                        const int gi = s + b + __ffs(fb) - 1;
                        fb &= fb - 1;
                        pair_fp64<DIM>(x, y, z, t.sx[gi], t.sy[gi], DIM == 3 ? t.sz[gi] : 0.0,
                                       t.sm[gi], eps2, a64);
                        cnt[4]++;
                    }
                }
                __syncwarp();
            }
            if (act) {   // renormalise the accumulators once per leaf
#pragma unroll
                for (int k = 0; k < DIM; k++) {
                    float hsum = __fadd_rn(ah[k], al[k]);
                    al[k] = __fsub_rn(al[k], __fsub_rn(hsum, ah[k]));
                    ah[k] = hsum;
                }
            }
        } else {
            bool open = false;
            float4 nh = make_float4(0.f, 0.f, 0.f, 0.f);
            if (act) {
                nh = ft.nh[node];
                const float4 nlo = ft.nl[node];
                float d2 = 0.0f;
#pragma unroll
                for (int k = 0; k < DIM; k++) {
                    // hi and lo differences (both exact inside the box), rounded once
                    float d = __fadd_rn(__fsub_rn(comp(nh, k), Th[k]), __fsub_rn(comp(nlo, k), Tl[k]));
                    d2 = fmaf(d, d, d2);
                }
                const float dist = d2 > 0.0f ? d2 * rsqrtf(d2) : 0.0f;
                const float td = theta_f * dist;
                const float band = theta_f * fmaf(kBandRel, dist, band_abs);
                const float size_f = __int_as_float(hd.y);
                if (size_f >= td + band) {
                    open = true;
                } else if (size_f < td - band) {
                    open = false;
                } else {
                    open = open_exact64<DIM>(x, y, z, t.cm[node], t.size[node], a.theta);
                    cnt[3] += lead;
                }
            }
            const unsigned omask = __ballot_sync(FULL, act && open);
            if (act && !open && lead) {
                const float4 nl = ft.nl[node];   // (cached: read by the opening test)
                if (!FAR && !CHECK) {
                    pair_ff_soft<DIM, false>(Th, Tl, nh, nl, a.e2h, a.e2l, ah, al);
                } else if (!pair_ff<DIM, FAR, CHECK>(Th, Tl, nh, nl, a.e2h, a.e2l, ah, al)) {
                    const NodeCM cm = t.cm[node];
                    pair_fp64<DIM>(x, y, z, cm.x, cm.y, cm.z, cm.w, eps2, a64);
                    cnt[4]++;
                }
                cnt[1]++;
            }
            if (omask) {
                if (sp + 2 > kStackDepth) { overflow = true; break; }
                if (lane == 0) {
                    stack[w][sp] = make_int2(fc, (int)omask);
                    stack[w][sp + 1] = make_int2(fc + 1, (int)omask);
                }
                sp += 2;
                __syncwarp();
            }
        }
    }
}

// SOFT: (eps s)^2 >= 2 kTinyR, so a warp of targets inside the box needs no
// small-R test (pair_ff's CHECK).
template <int DIM, bool SOFT>
__global__ void __launch_bounds__(kFastThreads, kFastBlocksPerSM)
k_traverse_fast(TreeDev t, FastTree ft, FastArgs a)
{
    __shared__ int2 stack[kFastWarps][kStackDepth];
    __shared__ float4 sh[kFastWarps][kWarp], sl[kFastWarps][kWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    const FastFrame fr = *ft.frame;
    const double conv = __dmul_rn(fr.conv, a.G);

    for (int64_t base = ((int64_t)blockIdx.x * kFastWarps + w) * kWarp; base < a.nt;
         base += (int64_t)gridDim.x * kFastWarps * kWarp) {
        const int64_t i = base + lane;
        const bool valid = i < a.nt;
        float Th[3] = {0.f, 0.f, 0.f}, Tl[3] = {0.f, 0.f, 0.f};
        bool far = false;
        float amax = 0.f;
        double x = 0.0, y = 0.0, z = 0.0;
        if (valid) {
            // self targets are the sorted particles themselves (inside the box)
            const float4 h = a.th ? a.th[i] : ft.ph[i];
            const float4 l = a.th ? a.tl[i] : ft.pl[i];
            Th[0] = h.x; Th[1] = h.y; Th[2] = h.z;
            Tl[0] = l.x; Tl[1] = l.y; Tl[2] = l.z;
            far = a.th ? h.w != 0.0f : false;
            amax = a.th ? l.w : 1.0f;
            x = a.tx[i];
            y = a.ty[i];
            z = DIM == 3 ? a.tz[i] : 0.0;
        }
        const float band_abs = kBandAbs * (1.0f + amax);
        float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};
        double a64[3] = {0.0, 0.0, 0.0};
        unsigned cnt[5] = {0, 0, 0, 0, 0};
        // self mode: targets are the sorted particles, target i is particle i
        const int64_t me_sorted = (valid && a.th == nullptr) ? i : -1;
        bool overflow = false;
        if (__any_sync(FULL, far))
            walk<DIM, true, true>(t, ft, a, w, lane, valid, me_sorted, Th, Tl, band_abs, x, y, z,
                                  ah, al, a64, stack, sh, sl, cnt, overflow);
        else if (SOFT && fr.unit)
            walk<DIM, false, false, true>(t, ft, a, w, lane, valid, me_sorted, Th, Tl, band_abs, x,
                                          y, z, ah, al, a64, stack, sh, sl, cnt, overflow);
        else
            walk<DIM, false, !SOFT>(t, ft, a, w, lane, valid, me_sorted, Th, Tl, band_abs, x, y, z,
                                    ah, al, a64, stack, sh, sl, cnt, overflow);
        if (overflow && lane == 0) atomicOr(a.err, kErrStackOverflow);
        if (a.stats) {
#pragma unroll
            for (int k = 0; k < 5; k++) {
                unsigned long long v = cnt[k];   // per-target counts fit 32 bits
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if (lane == 0 && v) atomicAdd(&a.stats[k], v);
            }
        }
        if (valid) {
            const int64_t o = a.out_idx ? a.out_idx[i] : i;
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                double v = __dadd_rn((double)ah[k], (double)al[k]);
                a.out[o * DIM + k] = __dadd_rn(__dmul_rn(v, conv), __dmul_rn(a64[k], a.G));
            }
        }
    }
}

// Self accelerations of few targets (fewer warps than two per SM
// sub-partition): LPT lanes per target, so that LPT times as many warps
// share the work (soft path only; the group's partial sums are added by
// shuffles in a fixed order at the end).
template <int DIM, int LPT>
__global__ void __launch_bounds__(kFastThreads, kFastBlocksPerSM)
k_traverse_fast_lpt(TreeDev t, FastTree ft, FastArgs a)
{
    constexpr int kTargets = kWarp / LPT;   // targets per warp
    __shared__ int2 stack[kFastWarps][kStackDepth];
    __shared__ float4 sh[kFastWarps][kWarp], sl[kFastWarps][kWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    const FastFrame fr = *ft.frame;
    const double conv = __dmul_rn(fr.conv, a.G);
    for (int64_t base = ((int64_t)blockIdx.x * kFastWarps + w) * kTargets; base < a.nt;
         base += (int64_t)gridDim.x * kFastWarps * kTargets) {
        const int64_t i = base + lane / LPT;
        const bool valid = i < a.nt;
        float Th[3] = {0.f, 0.f, 0.f}, Tl[3] = {0.f, 0.f, 0.f};
        double x = 0.0, y = 0.0, z = 0.0;
        if (valid) {
            const float4 h = ft.ph[i], l = ft.pl[i];
            Th[0] = h.x; Th[1] = h.y; Th[2] = h.z;
            Tl[0] = l.x; Tl[1] = l.y; Tl[2] = l.z;
            x = a.tx[i];
            y = a.ty[i];
            z = DIM == 3 ? a.tz[i] : 0.0;
        }
        const float band_abs = kBandAbs * 2.0f;
        float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};
        double a64[3] = {0.0, 0.0, 0.0};
        unsigned cnt[5] = {0, 0, 0, 0, 0};
        const int64_t me_sorted = valid ? i : -1;
        bool overflow = false;
        if (fr.unit)
            walk<DIM, false, false, true, LPT>(t, ft, a, w, lane, valid, me_sorted, Th, Tl,
                                               band_abs, x, y, z, ah, al, a64, stack, sh, sl, cnt,
                                               overflow);
        else
            walk<DIM, false, false, false, LPT>(t, ft, a, w, lane, valid, me_sorted, Th, Tl,
                                                band_abs, x, y, z, ah, al, a64, stack, sh, sl,
                                                cnt, overflow);
        if (overflow && lane == 0) atomicOr(a.err, kErrStackOverflow);
#pragma unroll
        for (int o = LPT / 2; o >= 1; o >>= 1) {
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                const float bh = __shfl_down_sync(FULL, ah[k], o);
                const float bl = __shfl_down_sync(FULL, al[k], o);
                ff_add(ah[k], al[k], bh, bl);
            }
        }
        if (a.stats) {
#pragma unroll
            for (int k = 0; k < 5; k++) {
                unsigned long long v = cnt[k];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if (lane == 0 && v) atomicAdd(&a.stats[k], v);
            }
        }
        if (valid && (lane & (LPT - 1)) == 0) {
            const int64_t o = a.out_idx ? a.out_idx[i] : i;
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                double v = __dadd_rn((double)ah[k], (double)al[k]);
                a.out[o * DIM + k] = __dmul_rn(v, conv);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// form "fp32": the precision form.  Pair terms, monopoles and the opening
// test in FP32 on hi + lo displacements (each difference exact, rounded
// once); per-target sums Kahan-compensated: every monopole, and every leaf
// block of at most 32 pair terms (summed in FP32 first), is one Kahan step.
// FP64 stays in the tree build (bounding box, Morton keys, masses and
// centres of mass, quadrupoles) and in the final scaling.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void walk_f32(const TreeDev& t, const FastTree& ft, const FastArgs& a,
                                         int w, int lane, bool valid, int64_t me_sorted,
                                         const float* T, const float* Tl, float* acc, float* cmp,
                                         int2 (*stack)[kStackDepth], float4 (*sh)[kWarp],
                                         float4 (*sl)[kWarp], unsigned* cnt, bool& overflow)
{
    const unsigned FULL = 0xffffffffu;
    const float theta_f = (float)a.theta;
    const bool soft = a.e2h >= 0x1p-126f;   // r^2 >= eps^2 is normal: no small-r test
    const bool unit = ft.frame->unit != 0;   // every particle mass exactly 1
    const TargetF32x2 tx = target_f32x2(T, Tl);
    const unsigned live = __ballot_sync(FULL, valid);
    if (lane == 0) stack[w][0] = make_int2(0, (int)live);
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int2 e = stack[w][--sp];
        __syncwarp();
        const int node = e.x;
        const unsigned mask = (unsigned)e.y;
        const bool act = (mask >> lane) & 1u;
        cnt[2] += act;
        const int4 hd = ft.nhdr[node];   // (first_child, start, count, mass != 0)
        if (!hd.w) continue;
        const int fc = hd.x;
        if (fc < 0) {
            const int s = hd.y, c = hd.z;
            for (int b = 0; b < c; b += kWarp) {
                const int jj = b + lane;
                if (jj < c) {
                    sh[w][lane] = ft.ph[s + jj];
                    sl[w][lane] = ft.pl[s + jj];
                }
                __syncwarp();
                const int cn = min(kWarp, c - b);
                if (act) {
                    cnt[0] += cn - (me_sorted >= s + b && me_sorted < s + b + cn);
                    float2 pxy = make_float2(0.f, 0.f);   // <= 32 terms, then one Kahan step
                    float pz = 0.f;
                    if (soft && unit) {
#pragma unroll (kF32Unroll)
                        for (int q = 0; q < cn; q++)
                            pair_f32_partial2<DIM, false, true>(tx, sh[w][q], sl[w][q], a.e2h,
                                                                pxy, pz);
                    } else if (soft) {
#pragma unroll (kF32Unroll)
                        for (int q = 0; q < cn; q++)
                            pair_f32_partial2<DIM, false, false>(tx, sh[w][q], sl[w][q], a.e2h,
                                                                 pxy, pz);
                    } else {
#pragma unroll (kF32Unroll)
                        for (int q = 0; q < cn; q++)
                            pair_f32_partial2<DIM, true, false>(tx, sh[w][q], sl[w][q], a.e2h,
                                                                pxy, pz);
                    }
                    const float part[3] = {pxy.x, pxy.y, pz};
                    kahan_add_f32<DIM>(part, acc, cmp);
                }
                __syncwarp();
            }
        } else {
            bool open = false;
            float4 nh = make_float4(0.f, 0.f, 0.f, 0.f);
            if (act) {
                // opening test on the hi coordinates (exact differences on
                // the 2^-23 grid): the FP32 form's criterion is a heuristic,
                // so a decision at the margin may go either way
                nh = ft.nh[node];
                float d2 = 0.0f;
#pragma unroll
                for (int k = 0; k < DIM; k++) {
                    const float d = __fsub_rn(comp(nh, k), T[k]);
                    d2 = fmaf(d, d, d2);
                }
                const float dist = d2 > 0.0f ? d2 * rsqrtf(d2) : 0.0f;
                const float size_f = __int_as_float(hd.y);
                if (a.mac == 1) {
                    // offset criterion: open when d < size/theta + |com - centre|
                    open = size_f >= theta_f * (dist - __int_as_float(hd.z));
                } else {
                    open = dist == 0.0f || size_f >= theta_f * dist;
                }
            }
            const unsigned omask = __ballot_sync(FULL, act && open);
            if (act && !open) {
                if (ft.nq0)
                    node_quad_f32<DIM>(T, Tl, nh, ft.nl[node], ft.nq0[node], ft.nq1[node], a.e2h,
                                       acc, cmp);
                else
                    pair_f32<DIM>(T, Tl, nh, ft.nl[node], a.e2h, acc, cmp);
                cnt[1]++;
            }
            if (omask) {
                if (sp + 2 > kStackDepth) { overflow = true; break; }
                if (lane == 0) {
                    stack[w][sp] = make_int2(fc, (int)omask);
                    stack[w][sp + 1] = make_int2(fc + 1, (int)omask);
                }
                sp += 2;
                __syncwarp();
            }
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(kFastThreads)
k_traverse_fp32(TreeDev t, FastTree ft, FastArgs a)
{
    __shared__ int2 stack[kFastWarps][kStackDepth];
    __shared__ float4 sh[kFastWarps][kWarp], sl[kFastWarps][kWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    const double conv = __dmul_rn(ft.frame->conv, a.G);
    for (int64_t base = ((int64_t)blockIdx.x * kFastWarps + w) * kWarp; base < a.nt;
         base += (int64_t)gridDim.x * kFastWarps * kWarp) {
        const int64_t i = base + lane;
        const bool valid = i < a.nt;
        float T[3] = {0.f, 0.f, 0.f}, Tl[3] = {0.f, 0.f, 0.f};
        if (valid) {
            const float4 h = a.th ? a.th[i] : ft.ph[i];
            const float4 l = a.th ? a.tl[i] : ft.pl[i];
            T[0] = h.x; T[1] = h.y; T[2] = h.z;
            Tl[0] = l.x; Tl[1] = l.y; Tl[2] = l.z;
        }
        float acc[3] = {0.f, 0.f, 0.f}, cmp[3] = {0.f, 0.f, 0.f};
        unsigned cnt[5] = {0, 0, 0, 0, 0};
        const int64_t me_sorted = (valid && a.th == nullptr) ? i : -1;
        bool overflow = false;
        walk_f32<DIM>(t, ft, a, w, lane, valid, me_sorted, T, Tl, acc, cmp, stack, sh, sl, cnt,
                      overflow);
        if (overflow && lane == 0) atomicOr(a.err, kErrStackOverflow);
        if (a.stats) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                unsigned long long v = cnt[k];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if (lane == 0 && v) atomicAdd(&a.stats[k], v);
            }
        }
        if (valid) {
            const int64_t o = a.out_idx ? a.out_idx[i] : i;
#pragma unroll
            for (int k = 0; k < DIM; k++)   // Kahan sum: value = sum - compensation
                a.out[o * DIM + k] = __dmul_rn(__dsub_rn((double)acc[k], (double)cmp[k]), conv);
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_fast_prepare(const double* box, int dim, FastFrame* frame, const TreeDev& t,
                        const double* center, float4* ph, float4* pl, float4* nh, float4* nl,
                        float* nsize, float* ndelta, const double* quad, float4* nq0,
                        float2* nq1, int4* nhdr, cudaStream_t s)
{
    k_frame<<<1, 32, 0, s>>>(box, dim, frame);
    k_ff_particles<<<grid_for(t.n, 256), 256, 0, s>>>(t.sx, t.sy, t.sz, t.sm, t.n, dim, frame, ph,
                                                      pl);
    k_ff_nodes<<<grid_for(t.m, 256), 256, 0, s>>>(t, center, frame, nh, nl, nsize, ndelta, quad,
                                                  nq0, nq1, nhdr);
    BHUT_CUDA(cudaGetLastError());
    note_launches(3);
    return kOk;
}

int launch_fast_targets(const double* tx, const double* ty, const double* tz, int64_t nt, int dim,
                        const FastFrame* frame, float4* th, float4* tl, cudaStream_t s)
{
    k_ff_targets<<<grid_for(nt, 256), 256, 0, s>>>(tx, ty, tz, nt, dim, frame, th, tl);
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

int launch_traverse_fast(const TreeDev& t, const FastTree& ft, const float4* th, const float4* tl,
                         const double* tx, const double* ty, const double* tz,
                         const int32_t* self_id, const int32_t* out_idx, int64_t nt, double theta,
                         double eps, double G, double eps_scaled_sq, double* out, unsigned* err,
                         unsigned long long* stats, cudaStream_t s, bool fp32, int mac)
{
    if (nt <= 0) return kOk;
    FastArgs a;
    a.th = th; a.tl = tl; a.tx = tx; a.ty = ty; a.tz = tz;
    a.self_id = self_id; a.out_idx = out_idx; a.nt = nt;
    a.theta = theta; a.eps = eps; a.G = G;
    a.e2h = (float)eps_scaled_sq;
    a.e2l = (float)(eps_scaled_sq - (double)a.e2h);
    a.out = out; a.err = err; a.stats = stats; a.mac = mac;
    int64_t warps = (nt + kWarp - 1) / kWarp;
    unsigned grid = grid_for(warps, kFastWarps, 152u * 64u);
    if (fp32) {
        if (t.dim == 3) k_traverse_fp32<3><<<grid, kFastThreads, 0, s>>>(t, ft, a);
        else k_traverse_fp32<2><<<grid, kFastThreads, 0, s>>>(t, ft, a);
    } else {
        const bool soft = a.e2h >= 2.0f * kTinyR;
        // few self targets: lanes per target so that about two warps run on
        // each SM sub-partition (self targets lie in the box: soft path)
        int lpt = 1;
        if (soft && th == nullptr && BHUT_FAST_MAX_LPT > 1) {
            int dev = 0, sms = 0;
            BHUT_CUDA(cudaGetDevice(&dev));
            BHUT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            const int64_t want = (int64_t)BHUT_FAST_LPT_WARPS_PER_SM * sms;
            while (lpt < BHUT_FAST_MAX_LPT && (nt * lpt + kWarp - 1) / kWarp < want) lpt *= 2;
        }
        if (lpt > 1) {
            const unsigned g = grid_for((nt * lpt + kWarp - 1) / kWarp, kFastWarps, 152u * 64u);
            if (t.dim == 3) {
                if (lpt == 2) k_traverse_fast_lpt<3, 2><<<g, kFastThreads, 0, s>>>(t, ft, a);
                else if (lpt == 4) k_traverse_fast_lpt<3, 4><<<g, kFastThreads, 0, s>>>(t, ft, a);
                else k_traverse_fast_lpt<3, 8><<<g, kFastThreads, 0, s>>>(t, ft, a);
            } else {
                if (lpt == 2) k_traverse_fast_lpt<2, 2><<<g, kFastThreads, 0, s>>>(t, ft, a);
                else if (lpt == 4) k_traverse_fast_lpt<2, 4><<<g, kFastThreads, 0, s>>>(t, ft, a);
                else k_traverse_fast_lpt<2, 8><<<g, kFastThreads, 0, s>>>(t, ft, a);
            }
        } else if (t.dim == 3) {
            if (soft) k_traverse_fast<3, true><<<grid, kFastThreads, 0, s>>>(t, ft, a);
            else k_traverse_fast<3, false><<<grid, kFastThreads, 0, s>>>(t, ft, a);
        } else {
            if (soft) k_traverse_fast<2, true><<<grid, kFastThreads, 0, s>>>(t, ft, a);
            else k_traverse_fast<2, false><<<grid, kFastThreads, 0, s>>>(t, ft, a);
        }
    }
    BHUT_CUDA(cudaGetLastError());
    note_launches(1);
    return kOk;
}

}  // namespace bhut
