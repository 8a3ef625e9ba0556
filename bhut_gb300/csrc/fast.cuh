// Device arithmetic shared by the single-tree and batched traversals:
// normalisation frames, the grid-aligned hi/lo split of coordinates, the
// float-float pair term (form "fast"), the FP32 pair term (form "fp32"),
// the FP64 pair term and the exact FP64 opening test used as fallbacks.
#pragma once
#include "tree.cuh"

// Accumulation two-sum of pair_ff_soft: 0 = FastTwoSum on the operands
// ordered by magnitude (ALU compare and selects), 1 = Knuth's TwoSum (six
// FP32 operations).  Both are exact; build-time switch for measurements.
#ifndef BHUT_FF_KNUTH_ACC
#define BHUT_FF_KNUTH_ACC 0
#endif
// Unroll factor of the float-float leaf pair loops (swept on GB300 at 1M
// Plummer: 4 beats 1-2 by 2-10 %).
#ifndef BHUT_FF_UNROLL
#define BHUT_FF_UNROLL 4
#endif

namespace bhut {

constexpr int kFFUnroll = BHUT_FF_UNROLL;
// leaf_block_soft: leaf visits with at most BHUT_SPLIT_MAXK active lanes are
// split across the idle lanes; the split pair loop is unrolled
// BHUT_SPLIT_UNROLL times.  Swept on GB300 at 1M Plummer (theta 0.5, leaf
// 32): split at <= 16 active lanes 173.8 ms, at <= 8 178.9 ms, no split
// 187.2 ms; split-loop unroll 2 173.8 ms, 1 174.0 ms, 4 175.7 ms.  The FP32
// form's pair term is too cheap for the split to pay (63.9-64.1 ms against
// 62.7 ms unsplit), so it keeps one lane per target.
#ifndef BHUT_SPLIT_MAXK
#define BHUT_SPLIT_MAXK 16
#endif
#ifndef BHUT_SPLIT_UNROLL
#define BHUT_SPLIT_UNROLL 2
#endif
constexpr int kSplitMaxK = BHUT_SPLIT_MAXK;
constexpr int kSplitUnroll = BHUT_SPLIT_UNROLL;
static_assert(kSplitMaxK <= 16, "a split gives every active target at least two lanes");

// The coordinates are represented to 2^-48 (normalised units), so a pair's
// relative error is about 2^-48 / sqrt(R), R = r^2 + eps^2.
// Softened path: every R is at least eps^2, and the range test is compiled
// out when (eps s)^2 >= 2 kTinyR.
constexpr float kTinyR = 0x1p-34f;
// Checked path (small or no softening): R below this -> FP64 pair, so a
// float-float pair's relative error stays below 2^-35.
constexpr float kTinyRCheck = 0x1p-26f;
constexpr float kHugeR = 0x1p+100f;    // r^2 above this -> FP64 pair
constexpr float kBandRel = 0x1p-18f;   // opening-test error band, relative part
constexpr float kBandAbs = 0x1p-40f;   // ... absolute part per unit of (1 + |target|)

static __device__ void frame_from_box(const double* box, int dim, FastFrame* f)
{
    double h = 0.0;
    for (int d = 0; d < 3; d++) f->c[d] = 0.0;
    for (int d = 0; d < dim; d++) {
        f->c[d] = __dmul_rn(__dadd_rn(box[d], box[3 + d]), 0.5);
        double e = __dmul_rn(__dsub_rn(box[3 + d], box[d]), 0.5);
        h = e > h ? e : h;
    }
    if (!(h > 0.0)) h = 1.0;
    // Map the box into [-1/2, 1/2]: a refit may move particles to 1.1x the
    // root box (bhut/tree/refit.py:236-249) and targets inside [-1, 1] are
    // still on the grid; every hi difference then stays below 2 and is exact.
    int ex;
    frexp(h, &ex);                      // h <= 2^ex
    f->s = ldexp(1.0, -ex - 1);
    double mm = box[6];
    int em = 0;
    if (mm > 0.0) frexp(mm, &em);       // |m| <= 2^em
    f->ms = ldexp(1.0, -em);
    f->conv = ldexp(1.0, em - 2 * ex - 2);  // normalised -> physical acceleration (s^2 / ms)
    f->unit = 0;
}

// Every particle has the same positive mass m0 (flag set by the
// bounding-box kernel): masses are measured in units of m0, so a particle's
// normalised mass is exactly 1 and a node's is M / m0 (FP64, then split hi +
// lo).
static __device__ void frame_unit_mass(double m0, bool uniform, FastFrame* f)
{
    if (!uniform || !(m0 > 0x1p-1000 && m0 < 0x1p+1000)) return;
    f->ms = __drcp_rn(m0);
    f->conv = __dmul_rn(__dmul_rn(m0, f->s), f->s);   // s a power of two: exact
    f->unit = 1;
}


// hi on the 2^-23 grid and lo on the 2^-47 grid (both exact in FP32 for
// |u| <= 1): differences of hi parts, and of lo parts, are then exact in
// FP32; u is represented to within 2^-48.
static __device__ __forceinline__ void split_grid(double u, float& h, float& l)
{
    double H = rint(__dmul_rn(u, 8388608.0));
    double hd = __dmul_rn(H, 1.0 / 8388608.0);
    h = __double2float_rn(hd);
    double L = rint(__dmul_rn(__dsub_rn(u, hd), 140737488355328.0));   // 2^47
    l = __double2float_rn(__dmul_rn(L, 1.0 / 140737488355328.0));
}

static __device__ __forceinline__ void split_plain(double u, float& h, float& l)
{
    h = __double2float_rn(u);
    l = __double2float_rn(__dsub_rn(u, (double)h));
}


// ---------------------------------------------------------------------------
// float-float pair term
// ---------------------------------------------------------------------------
// Error of s = fl(a + b) (Knuth's TwoSum).
static __device__ __forceinline__ float two_sum_err(float a, float b, float s)
{
    float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// MUFU reciprocal square root, flush-to-zero (one instruction; callers pass
// normal, positive arguments only).
static __device__ __forceinline__ float rsqrt_mufu(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

static __device__ __forceinline__ float comp(const float4& v, int k)
{
    return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

// Adds G-less m * (x_src - x_tgt) / (|dx|^2 + eps^2)^(3/2), normalised
// units, to (ah, al).  Returns false when the pair must go to FP64; it then
// adds exactly zero (the term is computed on a stand-in R and discarded with
// selects, so the pair loop has no branch).
//
// d = hi_src - hi_tgt is exact on the grid and l = lo_src - lo_tgt is small
// (|l| <= 2^-23), so (d, l) is renormalised with FastTwoSum into (gh, gl),
// |gl| <= ulp(gh) / 2; every later product of a float-float with g then
// keeps ~2^-47 relative accuracy.  A pair at zero displacement (the target
// itself, or a duplicate) contributes exactly zero, as in the reference.
//
// CHECK = false: the caller guarantees R >= kTinyR for every pair (a target
// inside the box and a softening with (eps s)^2 >= 2 kTinyR: R >= eps^2 up to
// the 2^-20 relative error of the error terms), so the test and its selects
// are compiled out and the result is the same bit for bit.
template <int DIM, bool FAR, bool CHECK = true>
__device__ __forceinline__ bool pair_ff(const float* Th, const float* Tl, float4 sh, float4 sl,
                                        float e2h, float e2l, float* ah, float* al)
{
    float gh[3], gl[3];
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float xh = comp(sh, k);
        const float d = __fsub_rn(xh, Th[k]);        // exact on the grid
        float l = __fsub_rn(comp(sl, k), Tl[k]);
        if (FAR) l = __fadd_rn(l, two_sum_err(xh, -Th[k], d));
        const float h = __fadd_rn(d, l);             // FastTwoSum(d, l), |l| <= |d| or d == 0
        gl[k] = __fsub_rn(l, __fsub_rn(h, d));
        gh[k] = h;
    }
    // R = |g|^2 + eps^2: squares error-free, cross terms 2 gh gl in FP32
    float s = __fmul_rn(gh[0], gh[0]);
    float lo = __fmaf_rn(gh[0], gh[0], -s);
    float c = __fmul_rn(gh[0], gl[0]);
#pragma unroll
    for (int k = 1; k < DIM; k++) {
        const float p = __fmul_rn(gh[k], gh[k]);
        const float q = __fmaf_rn(gh[k], gh[k], -p);
        const float t = __fadd_rn(s, p);
        lo = __fadd_rn(lo, __fadd_rn(two_sum_err(s, p, t), q));
        s = t;
        c = __fmaf_rn(gh[k], gl[k], c);
    }
    {
        const float t = __fadd_rn(s, e2h);
        lo = __fadd_rn(lo, __fadd_rn(two_sum_err(s, e2h, t), __fmaf_rn(2.0f, c, e2l)));
        s = t;
    }
    const float Rs = __fadd_rn(s, lo);
    // |dx| <= 2 inside the box: only FAR targets can exceed kHugeR
    const bool ok = FAR ? (Rs >= kTinyRCheck && Rs <= kHugeR) : (!CHECK || Rs >= kTinyRCheck);
    const float Rh = ok ? Rs : 1.0f;
    const float Rl = ok ? __fsub_rn(lo, __fsub_rn(Rs, s)) : 0.0f;
    // w = R^(-3/2): y ~ R^(-1/2); e = 1 - R y^2 exactly enough;
    // w = y^3 (1 - e)^(-3/2) = y^3 (1 + 3e/2 + 15e^2/8 + O(e^3))
    const float y = rsqrt_mufu(Rh);                  // Rh >= kTinyRCheck: normal
    const float Y = __fmul_rn(y, y);
    const float Ye = __fmaf_rn(y, y, -Y);
    const float e = -__fmaf_rn(Rh, Ye, __fmaf_rn(Rl, Y, __fmaf_rn(Rh, Y, -1.0f)));
    const float W = __fmul_rn(Y, y);
    const float We = __fmaf_rn(Ye, y, __fmaf_rn(Y, y, -W));
    const float corr = __fmul_rn(e, __fmaf_rn(1.875f, e, 1.5f));
    const float wh = W;
    const float wl = __fmaf_rn(W, corr, We);
    // f = m w (zero for a pair left to FP64)
    const float mh = ok ? sh.w : 0.0f, ml = ok ? sl.w : 0.0f;
    const float fh = __fmul_rn(mh, wh);
    const float fl = __fmaf_rn(mh, wl, __fmaf_rn(ml, wh, __fmaf_rn(mh, wh, -fh)));
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float Fh = __fmul_rn(fh, gh[k]);
        const float Fl = __fmaf_rn(fh, gl[k], __fmaf_rn(fl, gh[k], __fmaf_rn(fh, gh[k], -Fh)));
        const float t = __fadd_rn(ah[k], Fh);
        const float err = two_sum_err(ah[k], Fh, t);
        ah[k] = t;
        al[k] = __fadd_rn(al[k], __fadd_rn(err, Fl));
    }
    return ok;
}

// The float-float pair term for a target inside the box when the softening
// bounds R = |g|^2 + eps^2 from below ((eps s)^2 >= 2 kTinyR: no pair can go
// to FP64).  Same inputs and result as pair_ff<DIM, false, false> up to the
// last bits, with fewer operations:
//  * the squares and eps^2 are non-negative, so each of the three additions
//    of R's high part is Dekker's FastTwoSum on (max, min) (two min/max on
//    the ALU pipe and three FP32 operations instead of Knuth's six);
//  * R stays unnormalised as s + lo (|lo| <= 2^-22 s): the rsqrt is taken of
//    s and the correction term e = 1 - (s + lo) y^2 absorbs lo;
//  * w = y^3 (1 + 3e/2): |e| <= 2^-20.4 (MUFU error plus |lo| / s), so the
//    dropped 15e^2/8 term is below 2^-39.9 of the pair, and in practice far
//    below the 2^-48 representation of the coordinates (|g| is near-pair
//    sized: ~2^-36 relative for a leaf pair);
//  * the accumulation stays an exact two-sum, written as FastTwoSum on the
//    operands ordered by magnitude (one compare and two selects on the ALU
//    pipe, three FP32 operations);
//  * UNIT: masses are in units of the common particle mass (every particle
//    has mass exactly 1), so f = w and the mass product is skipped.
template <int DIM, bool UNIT>
__device__ __forceinline__ void pair_ff_soft(const float* Th, const float* Tl, float4 sh,
                                             float4 sl, float e2h, float e2l, float* ah, float* al)
{
    float gh[3], gl[3], p[3], q[3];
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float d = __fsub_rn(comp(sh, k), Th[k]);   // exact on the grid
        const float l = __fsub_rn(comp(sl, k), Tl[k]);   // exact on the lo grid
        const float h = __fadd_rn(d, l);                  // FastTwoSum(d, l)
        gl[k] = __fsub_rn(l, __fsub_rn(h, d));
        gh[k] = h;
        p[k] = __fmul_rn(h, h);
        q[k] = __fmaf_rn(h, h, -p[k]);                   // exact square error
    }
    float c = __fmul_rn(gh[0], gl[0]);
#pragma unroll
    for (int k = 1; k < DIM; k++) c = __fmaf_rn(gh[k], gl[k], c);
    // s = ((eps^2 + p0) + p1) + p2, each error exact
    float s = e2h, lo = __fmaf_rn(2.0f, c, e2l);
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float a = fmaxf(s, p[k]), b = fminf(s, p[k]);
        const float t = __fadd_rn(a, b);
        lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(b, __fsub_rn(t, a)), q[k]));
        s = t;
    }
    // y ~ s^(-1/2); A = (s + lo) y^2 - 1 = -e to ~2^-46
    const float y = rsqrt_mufu(s);                    // s >= eps^2 > 0: normal
    const float Y = __fmul_rn(y, y);
    const float Ye = __fmaf_rn(y, y, -Y);
    const float A = __fmaf_rn(s, Ye, __fmaf_rn(lo, Y, __fmaf_rn(s, Y, -1.0f)));
    const float W = __fmul_rn(Y, y);
    const float We = __fmaf_rn(Ye, y, __fmaf_rn(Y, y, -W));
    const float wl = __fmaf_rn(__fmul_rn(W, -1.5f), A, We);   // y^3 (1 + 1.5 e) - W
    float fh = W, fl = wl;
    if (!UNIT) {
        const float mh = sh.w, ml = sl.w;
        fh = __fmul_rn(mh, W);
        fl = __fmaf_rn(mh, wl, __fmaf_rn(ml, W, __fmaf_rn(mh, W, -fh)));
    }
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float Fh = __fmul_rn(fh, gh[k]);
        const float Fl = __fmaf_rn(fh, gl[k], __fmaf_rn(fl, gh[k], __fmaf_rn(fh, gh[k], -Fh)));
        const float t = __fadd_rn(ah[k], Fh);
#if BHUT_FF_KNUTH_ACC
        const float err = two_sum_err(ah[k], Fh, t);
#else
        const bool sw = fabsf(Fh) > fabsf(ah[k]);
        const float big = sw ? Fh : ah[k], small = sw ? ah[k] : Fh;
        const float err = __fsub_rn(small, __fsub_rn(t, big));
#endif
        ah[k] = t;
        al[k] = __fadd_rn(al[k], __fadd_rn(err, Fl));
    }
}

// Float-float (ah, al) += (bh, bl): TwoSum of the high parts, the low parts
// added to its error, renormalised by FastTwoSum.
static __device__ __forceinline__ void ff_add(float& ah, float& al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float e = __fadd_rn(two_sum_err(ah, bh, s), __fadd_rn(al, bl));
    const float h = __fadd_rn(s, e);
    al = __fsub_rn(e, __fsub_rn(h, s));
    ah = h;
}

// Position of the set bit of rank r (0-based, from the least significant
// bit) of m; m must have more than r bits set.
static __device__ __forceinline__ int nth_set_bit(unsigned m, int r)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc(m & ((1u << w) - 1u));
        if (r >= c) {
            r -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

// One block of cn <= 32 leaf particles, staged in sh/sl, for the targets of
// the lanes in `mask` (those that opened the leaf's parent), float-float
// soft path (pair_ff_soft).  Called by all 32 lanes.
//
// With more than 16 active lanes each lane adds its pairs in order to its
// accumulator.  With k <= 16 active lanes the idle lanes are put to work:
// every active target gets f lanes (f = 2..32, the largest power of two with
// f k <= 32); lane j works for the active target of rank j / f, on the pairs
// q = j mod f, j mod f + f, ..., into a float-float partial sum that starts
// at zero; the f partials are added in a fixed tree order (shuffles down by
// f/2, f/4, ..., 1) and the group's sum is added to the target's
// accumulator with ff_add.  Leaf visits with at most 16 active lanes carry
// most of the warp's idle lanes (a CPU replay of the walk at 1M Plummer,
// theta 0.5, leaf 32: 16 % of the leaf steps, 84 % of the idle lane-steps),
// and the split cuts the pair steps of a solve by about a tenth.  The order
// of every addition depends only on the mask and cn, so a result does not
// depend on which kernel (single tree or batched) evaluates it.
template <int DIM, bool UNIT>
__device__ __forceinline__ void leaf_block_soft(unsigned mask, int lane, const float* Th,
                                                const float* Tl, const float4* sh,
                                                const float4* sl, int cn, float e2h, float e2l,
                                                float* ah, float* al)
{
    const unsigned FULL = 0xffffffffu;
    const bool mine = (mask >> lane) & 1u;
    const int k = __popc(mask);
    if (k == 0) return;
    if (k > kSplitMaxK) {
        if (mine) {
#pragma unroll (kFFUnroll)
            for (int q = 0; q < cn; q++)
                pair_ff_soft<DIM, UNIT>(Th, Tl, sh[q], sl[q], e2h, e2l, ah, al);
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
    float ph[3] = {0.f, 0.f, 0.f}, pl[3] = {0.f, 0.f, 0.f};
    if (work) {
#pragma unroll (kSplitUnroll)
        for (int q = sub; q < cn; q += f)
            pair_ff_soft<DIM, UNIT>(T, L, sh[q], sl[q], e2h, e2l, ph, pl);
    }
    for (int o = f >> 1; o >= 1; o >>= 1) {
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            const float bh = __shfl_down_sync(FULL, ph[c], o);
            const float bl = __shfl_down_sync(FULL, pl[c], o);
            ff_add(ph[c], pl[c], bh, bl);
        }
    }
    const int leader = mine ? __popc(mask & ((1u << lane) - 1u)) * f : 0;
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const float gh = __shfl_sync(FULL, ph[c], leader);
        const float gl = __shfl_sync(FULL, pl[c], leader);
        if (mine) ff_add(ah[c], al[c], gh, gl);
    }
}

// FP64 pair in physical units, G-less (the Numba loop arithmetic).
template <int DIM>
__device__ __forceinline__ void pair_fp64(double x, double y, double z, double px, double py,
                                          double pz, double pm, double eps2, double* a64)
{
    const double dx = __dsub_rn(px, x), dy = __dsub_rn(py, y);
    const double dz = DIM == 3 ? __dsub_rn(pz, z) : 0.0;
    double r2 = __dmul_rn(dx, dx);
    r2 = __dadd_rn(r2, __dmul_rn(dy, dy));
    if (DIM == 3) r2 = __dadd_rn(r2, __dmul_rn(dz, dz));
    r2 = __dadd_rn(r2, eps2);
    if (r2 == 0.0) return;
    const double ri = __ddiv_rn(1.0, __dsqrt_rn(r2));
    const double f = __dmul_rn(pm, __dmul_rn(__dmul_rn(ri, ri), ri));
    a64[0] = __dadd_rn(a64[0], __dmul_rn(f, dx));
    a64[1] = __dadd_rn(a64[1], __dmul_rn(f, dy));
    if (DIM == 3) a64[2] = __dadd_rn(a64[2], __dmul_rn(f, dz));
}

// Exact opening test (bh.py:576-601), same arithmetic as k_traverse_exact.
template <int DIM>
__device__ __forceinline__ bool open_exact64(double x, double y, double z, const NodeCM& cm,
                                             double size, double theta)
{
    double dx = __dsub_rn(x, cm.x), dy = __dsub_rn(y, cm.y);
    double s;
    if (DIM == 3) {
        double dz = __dsub_rn(z, cm.z);
        s = __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
    } else {
        s = __fma_rn(dy, dy, __dmul_rn(dx, dx));
    }
    double d = __dsqrt_rn(s);
    if (d == 0.0) return true;
    return __ddiv_rn(size, d) >= theta;
}


// Displacement from the hi parts (exact on the grid) plus the lo parts
// (exact on their grid), rounded once: FP32-relative accuracy everywhere in
// the box, also in dense regions far from the box centre.
template <int DIM>
__device__ __forceinline__ void pair_f32(const float* Th, const float* Tl, float4 sh, float4 sl,
                                         float e2, float* acc, float* cmp)
{
    const float d0 = __fadd_rn(__fsub_rn(sh.x, Th[0]), __fsub_rn(sl.x, Tl[0]));
    const float d1 = __fadd_rn(__fsub_rn(sh.y, Th[1]), __fsub_rn(sl.y, Tl[1]));
    const float d2 = DIM == 3 ? __fadd_rn(__fsub_rn(sh.z, Th[2]), __fsub_rn(sl.z, Tl[2])) : 0.0f;
    float r2 = fmaf(d1, d1, fmaf(d0, d0, e2));
    if (DIM == 3) r2 = fmaf(d2, d2, r2);
    // r^2 + eps^2 == 0: no force (kernels.py:62-63); below the normal range
    // (closer than 2^-63 box sizes, unsoftened) the FP32 force would
    // overflow: none either.  Selected, not branched: f = 0 then.
    const bool ok = r2 >= 0x1p-126f;
    const float ri = rsqrt_mufu(ok ? r2 : 1.0f);
    const float f = ok ? sh.w * (ri * ri * ri) : 0.0f;
    const float d[3] = {d0, d1, d2};
#pragma unroll
    for (int k = 0; k < DIM; k++) {            // Kahan compensated sum
        const float y = fmaf(f, d[k], -cmp[k]);
        const float t = __fadd_rn(acc[k], y);
        cmp[k] = __fsub_rn(__fsub_rn(t, acc[k]), y);
        acc[k] = t;
    }
}


// FP32 pair term added to a plain FP32 partial sum p (no compensation): the
// leaf loop sums at most 32 such terms and then adds the partial to the
// Kahan-compensated per-target accumulator with kahan_add_f32 (blocked
// Kahan summation).  Same displacement, r^2 and force as pair_f32.
// CHECK = false: the caller guarantees e2 >= 2^-126; r^2 is an FMA chain of
// non-negative terms started at e2, so r^2 >= e2 and the test is compiled out
// (same result bit for bit).
template <int DIM, bool CHECK = true>
__device__ __forceinline__ void pair_f32_partial(const float* Th, const float* Tl, float4 sh,
                                                 float4 sl, float e2, float* p)
{
    const float d0 = __fadd_rn(__fsub_rn(sh.x, Th[0]), __fsub_rn(sl.x, Tl[0]));
    const float d1 = __fadd_rn(__fsub_rn(sh.y, Th[1]), __fsub_rn(sl.y, Tl[1]));
    const float d2 = DIM == 3 ? __fadd_rn(__fsub_rn(sh.z, Th[2]), __fsub_rn(sl.z, Tl[2])) : 0.0f;
    float r2 = fmaf(d1, d1, fmaf(d0, d0, e2));
    if (DIM == 3) r2 = fmaf(d2, d2, r2);
    const bool ok = !CHECK || r2 >= 0x1p-126f;
    const float ri = rsqrt_mufu(ok ? r2 : 1.0f);
    const float f = ok ? sh.w * (ri * ri * ri) : 0.0f;
    p[0] = fmaf(f, d0, p[0]);
    p[1] = fmaf(f, d1, p[1]);
    if (DIM == 3) p[2] = fmaf(f, d2, p[2]);
}

// A target's negated hi and lo coordinates, x and y packed for the f32x2
// instructions of pair_f32_partial2.
struct TargetF32x2 {
    float2 hxy, lxy;
    float hz, lz;
};

static __device__ __forceinline__ TargetF32x2 target_f32x2(const float* T, const float* Tl)
{
    TargetF32x2 t;
    t.hxy = make_float2(-T[0], -T[1]);
    t.lxy = make_float2(-Tl[0], -Tl[1]);
    t.hz = -T[2];
    t.lz = -Tl[2];
    return t;
}

// pair_f32_partial with the x and y components in Blackwell's f32x2
// instructions (FADD2 / FFMA2: two IEEE single operations per issue slot).
// Every operation and its order are those of pair_f32_partial (x - y is
// x + (-y) exactly), so the result is the same bit for bit.  UNIT: the
// source's mass is exactly 1 (the unit-mass frame) and the product with it
// is skipped, also exactly.
template <int DIM, bool CHECK, bool UNIT>
__device__ __forceinline__ void pair_f32_partial2(const TargetF32x2& t, float4 sh, float4 sl,
                                                  float e2, float2& pxy, float& pz)
{
    const float2 dxy = __fadd2_rn(__fadd2_rn(make_float2(sh.x, sh.y), t.hxy),
                                  __fadd2_rn(make_float2(sl.x, sl.y), t.lxy));
    const float dz = DIM == 3 ? __fadd_rn(__fadd_rn(sh.z, t.hz), __fadd_rn(sl.z, t.lz)) : 0.0f;
    float r2 = fmaf(dxy.y, dxy.y, fmaf(dxy.x, dxy.x, e2));
    if (DIM == 3) r2 = fmaf(dz, dz, r2);
    const bool ok = !CHECK || r2 >= 0x1p-126f;
    const float ri = rsqrt_mufu(ok ? r2 : 1.0f);
    const float w = ri * ri * ri;
    const float f = ok ? (UNIT ? w : sh.w * w) : 0.0f;
    pxy = __ffma2_rn(make_float2(f, f), dxy, pxy);
    if (DIM == 3) pz = fmaf(f, dz, pz);
}

template <int DIM>
__device__ __forceinline__ void kahan_add_f32(const float* p, float* acc, float* cmp)
{
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float y = __fsub_rn(p[k], cmp[k]);
        const float t = __fadd_rn(acc[k], y);
        cmp[k] = __fsub_rn(__fsub_rn(t, acc[k]), y);
        acc[k] = t;
    }
}

// A node's monopole plus its Plummer-softened traceless quadrupole (FP32
// form, multipole "quad"), Kahan-added.  With d = com - x (target to node),
// r^2 = |d|^2 + eps^2:
//   a = M d / r^3 - Q d / r^5 + (5/2) (d . Q d) d / r^7,
// the gradient of the potential -M/r - (1/2) d.Q d / r^5.
template <int DIM>
__device__ __forceinline__ void node_quad_f32(const float* Th, const float* Tl, float4 nh,
                                              float4 nl, float4 q0, float2 q1, float e2,
                                              float* acc, float* cmp)
{
    const float d0 = __fadd_rn(__fsub_rn(nh.x, Th[0]), __fsub_rn(nl.x, Tl[0]));
    const float d1 = __fadd_rn(__fsub_rn(nh.y, Th[1]), __fsub_rn(nl.y, Tl[1]));
    const float d2 = DIM == 3 ? __fadd_rn(__fsub_rn(nh.z, Th[2]), __fsub_rn(nl.z, Tl[2])) : 0.0f;
    float r2 = fmaf(d1, d1, fmaf(d0, d0, e2));
    if (DIM == 3) r2 = fmaf(d2, d2, r2);
    if (!(r2 >= 0x1p-126f)) return;
    const float ri = rsqrt_mufu(r2);
    const float ri2 = ri * ri;
    const float ri3 = ri2 * ri;
    const float ri5 = ri3 * ri2;
    const float qx = fmaf(q1.x, d2, fmaf(q0.w, d1, q0.x * d0));
    const float qy = fmaf(q1.y, d2, fmaf(q0.y, d1, q0.w * d0));
    const float qz = fmaf(q0.z, d2, fmaf(q1.y, d1, q1.x * d0));
    const float dqd = fmaf(d2, qz, fmaf(d1, qy, d0 * qx));
    const float f = fmaf(2.5f * dqd, ri5 * ri2, nh.w * ri3);
    const float d[3] = {d0, d1, d2}, q[3] = {qx, qy, qz};
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const float y = __fsub_rn(fmaf(f, d[k], -ri5 * q[k]), cmp[k]);
        const float t = __fadd_rn(acc[k], y);
        cmp[k] = __fsub_rn(__fsub_rn(t, acc[k]), y);
        acc[k] = t;
    }
}

}  // namespace bhut
