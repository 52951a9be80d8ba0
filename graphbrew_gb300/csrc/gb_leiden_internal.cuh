// gb_leiden_internal.cuh -- device helpers shared by the local-moving engines.
#pragma once

#include <cmath>
#include <vector>

#include "gb_common.cuh"

namespace gb {

constexpr int kWarpMaxDeg = 512;       // warp path up to this degree
constexpr int kWarpHash = 1024;        // per-warp shared table slots (>= 2 x kWarpMaxDeg)
constexpr int kHubThreads = 512;
constexpr int kHubSmemSlots = 16384;   // hub table in shared memory up to 8192 neighbours

__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
    return (uint32_t)(((uint64_t)x * 0x9E3779B97F4A7C15ull) >> 32);
}

// deltaModularity (:1295-1298) with the reference's association.
__device__ __forceinline__ double delta_q(double kuc, double kud, double ku, double sc, double sd, double M, double R) {
    const double a = __ddiv_rn(__dsub_rn(kuc, kud), M);
    const double t = __dadd_rn(__dsub_rn(sc, sd), ku);
    const double b = __dmul_rn(__dmul_rn(R, ku), t);
    const double den = __dmul_rn(__dmul_rn(2.0, M), M);
    return __dsub_rn(a, __ddiv_rn(b, den));
}

// The two divisors of deltaModularity for one graph, with double-double
// reciprocals, so that a candidate's quotients cost a few multiply-adds
// instead of two full divisions (this GPU's FP64 rate is low, and the
// evaluation kernels spend most of their issue slots on FP64).
constexpr int kAtabMax = 1024;   // RN(k / M) tabulated for 0 <= k <= kAtabMax

struct DqConst {
    double M = 1.0, R = 1.0;
    double den = 2.0;            // (2 M) M, formed as the reference forms it
    double yMh = 1.0, yMl = 0.0; // 1/M   ~ yMh + yMl
    double yDh = 0.5, yDl = 0.0; // 1/den ~ yDh + yDl
    const double* atab = nullptr;  // device: RN(k / M), k = 0..kAtabMax (fill_atab), or null
};

// Fills the device table tab[k] = RN(k / M), k = 0..kAtabMax, by full double
// divisions: (kuc - kud) / M of a row with at most kAtabMax neighbours in
// either community is then one load.
void fill_atab(double* tab, double M, cudaStream_t s);

// Host side: yh = RN(1/m); the remainder e = 1 - yh m is exact (the
// remainder of a correctly rounded quotient is representable), and
// yl = RN(e yh) leaves |yh + yl - 1/m| <= 2.01 * 2^-106 / m.
inline DqConst make_dq(double M, double R) {
    DqConst q;
    q.M = M;
    q.R = R;
    q.den = (2.0 * M) * M;
    auto recip = [](double m, double& h, double& l) {
        if (!(m > 0.0) || !std::isfinite(m)) { h = 0.0; l = 0.0; return; }
        h = 1.0 / m;
        l = std::fma(-h, m, 1.0) * h;
    };
    recip(q.M, q.yMh, q.yMl);
    recip(q.den, q.yDh, q.yDl);
    return q;
}

// RN(x / m) for a normal m > 0, given y = yh + yl within 2.01 * 2^-106 / m of
// 1/m, for x = 0 or 2^-900 < |x| < 2^900 (the integer and integer-times-R
// numerators of deltaModularity).  Written from the mathematics:
//  1. q = RN(|x| yh + RN(|x| yl)) is within |z| * 3.1 * 2^-106 of z = |x|/m
//     before its final rounding, so q is one of the two doubles around z
//     (a faithful quotient);
//  2. for a faithful quotient the remainder |x| - q m is a double (the
//     classical exact-remainder property of FMA division), so one FMA gives
//     it exactly, and its sign says on which side of q the quotient lies;
//  3. RN(z) is q or that neighbour: compare |r| with m times half the gap
//     between them (an exponent shift of m, exact).  A quotient of two
//     doubles never falls exactly on a midpoint, so no tie can occur; an
//     equal comparison would round to even.
// The result equals __ddiv_rn(x, m) bit for bit over that range (the
// self-check entry point gbgpu_selfcheck_delta compares both on the device).
__device__ __forceinline__ double div_rn_by(double x, double m, double yh, double yl) {
    const double ax = fabs(x);
    const double q = __fma_rn(ax, yh, __dmul_rn(ax, yl));
    const double r = __fma_rn(-q, m, ax);
    long long qb = __double_as_longlong(q);
    const long long rb = __double_as_longlong(r);
    const long long rmag = rb & 0x7FFFFFFFFFFFFFFFll;
    if (rmag != 0) {
        const bool up = rb > 0;                       // z above q
        const int e = (int)((qb >> 52) & 0x7FF);      // biased exponent of q
        // half the gap: 2^(e-1023-53) above q; below a power of two, half that
        int sh = e - 1076;
        if (!up && (qb & 0xFFFFFFFFFFFFFll) == 0) sh -= 1;
        const long long hb = __double_as_longlong(m) + ((long long)sh << 52);
        if (rmag > hb || (rmag == hb && (qb & 1))) qb += up ? 1 : -1;
    }
    return __longlong_as_double(qb | (__double_as_longlong(x) & (long long)0x8000000000000000ull));
}

// deltaModularity (:1295-1298) from integer counts: kuc and kud are the
// vertex's edges into c and into its own community d, ku its degree, sc and
// sd the two totals.  Every intermediate the reference rounds is rounded the
// same way: kuc - kud and sc - sd + ku are exact (integers below 2^53),
// R ku and R ku t are the reference's products, and the two quotients are
// correctly rounded by div_rn_by, so the value is bit-identical to delta_q.
__device__ __forceinline__ double delta_qi(const DqConst& q, long long kuc, long long kud, long long ku,
                                           long long sc, long long sd) {
    // RN(-k / M) = -RN(k / M): round-to-nearest is symmetric.
    const long long dk = kuc - kud, adk = dk < 0 ? -dk : dk;
    double a;
    if (adk <= kAtabMax && q.atab) {
        a = __ldg(q.atab + adk);
        if (dk < 0) a = -a;
    } else {
        a = div_rn_by((double)dk, q.M, q.yMh, q.yMl);
    }
    const double b = __dmul_rn(__dmul_rn(q.R, (double)ku), (double)(sc - sd + ku));
    return __dsub_rn(a, div_rn_by(b, q.den, q.yDh, q.yDl));
}

// d > 0.0 for a delta that is not NaN, on the integer pipe: a double is
// above +0.0 exactly when its bit pattern, read as a signed integer, is.
__device__ __forceinline__ bool dpos(double d) { return __double_as_longlong(d) > 0; }

// (delta, id) ordering: larger delta first, then smaller id.
__device__ __forceinline__ bool better(double da, uint32_t ia, double db, uint32_t ib) {
    return da > db || (da == db && ia < ib);
}

__device__ __forceinline__ void warp_argmax(double& d, uint32_t& c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xFFFFFFFFu, d, o);
        const uint32_t oc = __shfl_xor_sync(0xFFFFFFFFu, c, o);
        if (better(od, oc, d, c)) { d = od; c = oc; }
    }
}

// The same ordering for values that are +0.0 or positive (a selection that
// starts at +0.0 and only takes deltas > 0): such doubles order as their bit
// patterns, so the comparison runs on the integer pipe.
__device__ __forceinline__ bool better_pos(double da, uint32_t ia, double db, uint32_t ib) {
    const long long x = __double_as_longlong(da), y = __double_as_longlong(db);
    return x > y || (x == y && ia < ib);
}

__device__ __forceinline__ void warp_argmax_pos(double& d, uint32_t& c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xFFFFFFFFu, d, o);
        const uint32_t oc = __shfl_xor_sync(0xFFFFFFFFu, c, o);
        if (better_pos(od, oc, d, c)) { d = od; c = oc; }
    }
}

// Shared-memory open-addressing insert (keys kNone = empty).
__device__ __forceinline__ void table_add(uint32_t* keys, uint32_t* vals, uint32_t mask, uint32_t k, uint32_t w) {
    uint32_t h = hash_u32(k) & mask;
    while (true) {
        const uint32_t prev = atomicCAS(&keys[h], kNone, k);
        if (prev == kNone || prev == k) {
            atomicAdd(&vals[h], w);
            return;
        }
        h = (h + 1) & mask;
    }
}

__device__ __forceinline__ uint32_t table_get(const uint32_t* keys, const uint32_t* vals, uint32_t mask, uint32_t k) {
    uint32_t h = hash_u32(k) & mask;
    while (true) {
        const uint32_t s = keys[h];
        if (s == k) return vals[h];
        if (s == kNone) return 0;
        h = (h + 1) & mask;
    }
}


// State shared by the asynchronous and the exact local-moving engines.
struct LocalMoveContext {
    DeviceCSR g;
    uint32_t* vcom = nullptr;
    unsigned long long* ctot = nullptr;   // int64 totals (two's complement adds)
    uint8_t* vaff = nullptr;
    const uint32_t* vcob = nullptr;       // refinement bounds: localMovingPhase<true> when set
    double M = 1.0, R = 1.0;
    DqConst dq;
    std::vector<uint32_t> hubs_h;         // vertices above kWarpMaxDeg, id order
    const uint32_t* hubs = nullptr;
    int hub_grid = 1;
    uint32_t* hub_gk = nullptr;           // per-CTA global tables for very large hubs
    uint32_t* hub_gv = nullptr;
    int64_t hub_gcap = 0;
};

// Serial-order local moving (leiden_exact.cu).  Returns the iterations run.
int local_move_exact(const LocalMoveContext& ctx, double tolerance, int max_iterations, int64_t window,
                     cudaStream_t s, int64_t* launches, int64_t* rounds_out, int64_t* evals_out);

}  // namespace gb
