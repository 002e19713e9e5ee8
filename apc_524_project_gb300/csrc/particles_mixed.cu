// particles_mixed.cu - the mixed-precision form of the time loop.
//
// Particle state, 28 bytes per particle (structure of arrays):
//   cell    int32  linear index of the particle's cell in the (n+3)^3 field
//                  layout, cell = ix*sx + iy*sy + iz with ix in [1, n] (the
//                  reference's ghost-offset cell numbering)
//   ox..oz  float  in-cell offset in [0, 1) cell widths (split precision:
//                  position = x0 + d * (ix - 1 + o), exact to 2^-24 cells
//                  anywhere in the box)
//   ux..uz  float  momentum per unit mass, u = gamma v (v for the
//                  non-relativistic pusher)
// Fields E, B and B_tm1 are FP32 in the reference layout; J and rho are int64
// fixed-point values (quantum q0 = max_s |UNIT_RHOJ q_s / V| * 2^-32).
// Each warp sums the 20 contributions of consecutive particles that share a
// cell in FP32 in particle order, rounds each run total to the fixed-point
// quantum and adds it with integer atomics to that cell's 20 slots (one
// 160-byte record per cell, so a run commits in one coalesced instruction);
// a gather pass then forms J and rho at every point from the slots of its
// neighbour cells. Integer addition is associative, so J and rho are
// bit-reproducible.
//
// The arithmetic is the reference's algorithm (including its in-cell offset
// convention, Jx index, ghost and B-role behaviour, see the FP64 kernels) in
// FP32 with fused multiply-adds allowed. FP64 is kept for the Jacobi Poisson
// start (done on the FP64 grid slots, then converted), the Gauss-law check and
// the energy / momentum reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "dev_common.cuh"
#include "ad_mixed.cuh"
#include "emoo_internal.h"

namespace emoo {

struct FieldsF32 {
    float *E[3] = {nullptr, nullptr, nullptr};
    float *Bslot[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // BX..BZ, BX_TM1..BZ_TM1 storage
    long long *J[4] = {nullptr, nullptr, nullptr, nullptr};                    // Jx, Jy, Jz, rho
    double q0 = 1.0;  // fixed-point quantum
    float4 *pack = nullptr;  // interpolation pack, 5 float4 per grid point (interior cells filled)
    unsigned long long *wj = nullptr;  // per-cell J deposit sums, 12 int64 per grid point
    unsigned long long *wr = nullptr;  // per-cell rho deposit sums, 8 int64 per grid point
};

namespace {

constexpr float FOURPI_F = (float)(4.0 * PI_D);

struct MState {
    int32_t *cell;
    float *ox, *oy, *oz, *ux, *uy, *uz;
};

struct MSpecies {
    int nspec;
    int64_t off[EMOO_NSPEC + 1];
    float qp[EMOO_NSPEC];    // ((0.5 dt q)/m) UNIT_ACC
    float qdep[EMOO_NSPEC];  // (UNIT_RHOJ q / V) / q0: fixed-point units per unit weight and speed
    float m[EMOO_NSPEC];
    int deposit[EMOO_NSPEC];
};

__device__ __forceinline__ int species_of_m(const MSpecies &st, int64_t p) {
    int s = 0;
    while (s + 1 < st.nspec && p >= st.off[s + 1]) s++;
    return s;
}

struct MGeom {
    int n[3];
    int wrap[3];  // 1: the dimension is periodic (pieces of a path wrap); 0: walled
    int64_t sx, sy;
    int64_t npts;
    float dtid[3];  // dt / d
    float idf[3];   // 1 / d
    float ddt[3];   // d / dt (0 when dt = 0)
    float fourpi_dt;
};

struct FastDiv {  // floor(a / d) for 0 <= a < 2^31 via multiply-high
    uint32_t d, m;
    int s;
};

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1ull << l) < d) l++;
    f.s = l;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t a, const FastDiv &f) {
    uint32_t t = __umulhi(a, f.m);
    return (t + ((a - t) >> 1)) >> (f.s - 1 < 0 ? 0 : f.s - 1);
}

struct Div3 {
    FastDiv sx, sy;
};

__device__ __forceinline__ void split_cell(const MGeom &g, const Div3 &dv, int32_t c, int &ix, int &iy, int &iz) {
    uint32_t uc = (uint32_t)c;
    uint32_t i = (dv.sx.d == 1) ? uc : fdiv(uc, dv.sx);
    uint32_t r = uc - i * (uint32_t)g.sx;
    uint32_t j = (dv.sy.d == 1) ? r : fdiv(r, dv.sy);
    ix = (int)i;
    iy = (int)j;
    iz = (int)(r - j * (uint32_t)g.sy);
}

struct MGather {
    const float *E[3];
    const float *B[3];
    const float *T[3];
};

struct MDeposit {
    unsigned long long *wj;  // per-cell J sums, DEP_JSLOTS per cell
    unsigned long long *wr;  // per-cell rho sums, DEP_RSLOTS per cell
};

constexpr int DEP_SLOTS = 20;  // contributions per particle: J 12, rho 8
constexpr int DEP_JSLOTS = 12, DEP_RSLOTS = 8;

// Round-to-nearest-even of v as int64, the value of __float2ll_rn(v), without
// the float-to-int64 conversion: conversions run on the FP64 pipe, which on
// this GPU issues 2 lanes per clock per SM. Two exact FP32 steps split
// v = h 2^22 + l with |l| <= 2^21, and adding 1.5 * 2^23 (in the binade where
// the float spacing is 1) leaves each part's nearest integer in the low
// mantissa bits; h 2^22 is even, so the parts round as v does. Exact for
// |v| < 2^43; larger values (and NaN) take the conversion.
// GUARD = false drops the range test where |v| < 2^43 is known (see the
// relativistic deposit, where |velocity| < 1 bounds every run total).
template <bool GUARD = true>
__device__ __forceinline__ long long f2ll_rn(float v) {
    if (GUARD && !(fabsf(v) < 8.0e12f)) return __float2ll_rn(v);
    const float M = 12582912.0f;                    // 1.5 * 2^23
    const float hm = v * 2.384185791015625e-07f + M;  // M + rint(v 2^-22); v 2^-22 is exact
    const float lo = fmaf(M - hm, 4194304.0f, v);   // v - rint(v 2^-22) 2^22, exact
    const int hi = __float_as_int(hm) - __float_as_int(M);
    const int li = __float_as_int(lo + M) - __float_as_int(M);
    return ((long long)hi << 22) + li;
}

// New in-cell offset and cell index from the moved offset n (cell units):
// o = n - floor(n), i += floor(n). Moves of at most one cell are resolved by
// comparisons, which give the same values as floorf and keep the conversion
// instructions (FP64 pipe) out of the per-particle path.
__device__ __forceinline__ void cell_step(float n, int &i, float &o) {
    float f;
    if (n >= -1.0f && n < 2.0f) {
        const bool up = n >= 1.0f, down = n < 0.0f;
        f = up ? 1.0f : (down ? -1.0f : 0.0f);
        i += up ? 1 : (down ? -1 : 0);
    } else {
        f = floorf(n);
        i += (int)f;
    }
    o = n - f;
    // the subtraction can round to exactly 1.0f for tiny negative n
    if (o >= 1.0f) {
        o = 0.0f;
        i += 1;
    }
}

// Offset from the particle's cell of each of the 20 contribution points -
// Jx (4), Jy (4), Jz (4), rho (8) - as the FP64 deposit's table
// (src/grid/oGrid.cpp:98-111, 129-136; the Jx quirk at index 3), 3 bits per
// point (x: 4, y: 2, z: 1), point q at bits 3q..3q+2. A register constant,
// so lanes index it without a local-memory copy.
constexpr unsigned long long DEP_CODE =
    (0ull << 0) | (2ull << 3) | (3ull << 6) | (2ull << 9) |       // Jx: o, o+sy, o+sy+1, o+sy
    (0ull << 12) | (1ull << 15) | (5ull << 18) | (4ull << 21) |   // Jy: o, o+1, o+sx+1, o+sx
    (0ull << 24) | (4ull << 27) | (6ull << 30) | (2ull << 33) |   // Jz: o, o+sx, o+sx+sy, o+sy
    (0ull << 36) | (4ull << 39) | (6ull << 42) | (2ull << 45) |   // rho
    (3ull << 48) | (7ull << 51) | (5ull << 54) | (1ull << 57);

__host__ __device__ __forceinline__ int dep_offset(int q, int sx, int sy) {
    const int c = (int)((DEP_CODE >> (3 * q)) & 7ull);
    return (c >> 2) * sx + ((c >> 1) & 1) * sy + (c & 1);
}

// Position of contribution q in its cell's record. J (q < 12) and rho
// (q >= 12) have records of their own (rho is deposited only when asked
// for), each ordered by the point offset its slots feed:
//   J:   [0,3) offset 0: q 0 4 8 | [3,6) sy: q 1 3 11 | 6 1: q 5 | 7 sy+1: q 2
//        | 8 sx+1: q 6 | 9 sx+sy: q 10 | [10,12) sx: q 7 9
//   rho: 0 offset 0: q 12 | 1 sy: q 15 | 2 1: q 19 | 3 sy+1: q 16 | 4 sx+1: q 18
//        | 5 sx+sy: q 14 | 6 sx: q 13 | 7 sx+sy+1: q 17
// so a point gathers a neighbour's slots with few (vector) loads. 4 bits per q.
constexpr unsigned long long DEP_JPOS =  // q = 0..11
    (0ull << 0) | (3ull << 4) | (7ull << 8) | (4ull << 12) | (1ull << 16) | (6ull << 20) | (8ull << 24) |
    (10ull << 28) | (2ull << 32) | (11ull << 36) | (9ull << 40) | (5ull << 44);
constexpr unsigned long long DEP_RPOS =  // q = 12..19
    (0ull << 0) | (6ull << 4) | (5ull << 8) | (1ull << 12) | (3ull << 16) | (7ull << 20) | (4ull << 24) |
    (2ull << 28);

__host__ __device__ __forceinline__ int dep_pos(int q) {
    return q < 12 ? (int)((DEP_JPOS >> (4 * q)) & 15ull) : (int)((DEP_RPOS >> (4 * (q - 12))) & 15ull);
}

// The record layouts and the gather in k_cells_to_points must agree with the
// deposit table: every slot feeds the point offset of the q placed in it.
// Checked once per handle.
bool dep_tables_agree() {
    const int sx = 1000, sy = 30;  // distinct sums for all 8 offsets
    const int joff[DEP_JSLOTS] = {0, 0, 0, sy, sy, sy, 1, sy + 1, sx + 1, sx + sy, sx, sx};
    const int roff[DEP_RSLOTS] = {0, sy, 1, sy + 1, sx + 1, sx + sy, sx, sx + sy + 1};
    bool usedj[DEP_JSLOTS] = {}, usedr[DEP_RSLOTS] = {};
    for (int q = 0; q < DEP_SLOTS; q++) {
        const int pos = dep_pos(q);
        const bool j = q < 12;
        if (pos < 0 || pos >= (j ? DEP_JSLOTS : DEP_RSLOTS)) return false;
        bool &used = j ? usedj[pos] : usedr[pos];
        if (used || (j ? joff[pos] : roff[pos]) != dep_offset(q, sx, sy)) return false;
        used = true;
    }
    return true;
}

// ---- interpolation pack --------------------------------------------------
//
// The reference's gather (src/grid/oGrid.cpp:153-197 with
// src/particles/interpolate.cpp:11-47) uses the ghost-offset vertex, so the
// weights over an in-cell offset o are a = 2 - o and b = o - 1. An edge
// component interpolated over the offsets (t, r) of its two transverse axes is
//   a_t a_r F00 + b_t a_r F10 + b_t b_r F11 + a_t b_r F01
//     = c0 + ct t + cr r + ctr t r
// with the coefficients below, and the face component of B averaged with
// B_tm1 over its own axis offset s is
//   0.5 (a_s S0 + b_s S1) = d0 + d1 s,   S = B + B_tm1.
// The pack holds these 18 numbers per cell in 5 float4 (80 bytes):
//   [0] Ex c0 ct cr ctr (t = y, r = z)   [1] Ey (t = z, r = x)
//   [2] Ez (t = x, r = y)                [3] Bx d0 d1, By d0 d1
//   [4] Bz d0 d1, 2 unused
// so a particle reads 5 vector loads from one place instead of 24 scalars
// from 9 arrays. The pack is rebuilt from the fields before every push.
constexpr int PACK_F4 = 5;

__device__ __forceinline__ float4 edge_coef(float f00, float f10, float f11, float f01) {
    float4 c;
    c.x = (4.0f * f00 - 2.0f * f01) + (f11 - 2.0f * f10);
    c.y = (2.0f * f10 - 2.0f * f00) + (f01 - f11);
    c.z = (2.0f * f01 - 2.0f * f00) + (f10 - f11);
    c.w = (f00 - f10) + (f11 - f01);
    return c;
}

// The corrected policy's weights over the cell's own lower corner,
// a = 1 - o and b = o: the edge polynomial's coefficients, and for a face
// component 0.5 ((1 - s) S0 + s S1) = d0 + d1 s.
__device__ __forceinline__ float4 edge_coef_true(float f00, float f10, float f11, float f01) {
    return make_float4(f00, f10 - f00, f01 - f00, (f00 - f10) + (f11 - f01));
}

template <bool CORR>
__global__ void k_pack_m(MGeom g, MGather P, float4 *__restrict__ pack) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    const int64_t sx = g.sx, sy = g.sy;
    const int64_t o = (int64_t)i * sx + (int64_t)j * sy + k;
    const float *Ex = P.E[0], *Ey = P.E[1], *Ez = P.E[2];
    float4 *dst = pack + o * PACK_F4;
    auto coef = [](float f00, float f10, float f11, float f01) {
        return CORR ? edge_coef_true(f00, f10, f11, f01) : edge_coef(f00, f10, f11, f01);
    };
    // face term: d0 = S0 - S1/2 over the ghost-offset vertex, S0/2 over the true one
    auto d0 = [](float s0, float s1) { return CORR ? 0.5f * s0 : s0 - 0.5f * s1; };
    dst[0] = coef(Ex[o], Ex[o + sy], Ex[o + sy + 1], Ex[o + 1]);
    dst[1] = coef(Ey[o], Ey[o + 1], Ey[o + sx + 1], Ey[o + sx]);
    dst[2] = coef(Ez[o], Ez[o + sx], Ez[o + sx + sy], Ez[o + sy]);
    float s0, s1;
    float4 b;
    s0 = P.T[0][o] + P.B[0][o];
    s1 = P.T[0][o + sx] + P.B[0][o + sx];
    b.x = d0(s0, s1);
    b.y = 0.5f * (s1 - s0);
    s0 = P.T[1][o] + P.B[1][o];
    s1 = P.T[1][o + sy] + P.B[1][o + sy];
    b.z = d0(s0, s1);
    b.w = 0.5f * (s1 - s0);
    dst[3] = b;
    s0 = P.T[2][o] + P.B[2][o];
    s1 = P.T[2][o + 1] + P.B[2][o + 1];
    dst[4] = make_float4(d0(s0, s1), 0.5f * (s1 - s0), 0.0f, 0.0f);
}

// E and B at offsets (ox, oy, oz) of the cell whose pack starts at pk.
__device__ __forceinline__ void gather_pack(const float4 *__restrict__ pk, float ox, float oy, float oz, float f[6]) {
    const float4 ex = __ldg(pk), ey = __ldg(pk + 1), ez = __ldg(pk + 2), bxy = __ldg(pk + 3);
    const float2 bz = __ldg(reinterpret_cast<const float2 *>(pk + 4));
    f[0] = fmaf(oy, fmaf(oz, ex.w, ex.y), fmaf(oz, ex.z, ex.x));
    f[1] = fmaf(oz, fmaf(ox, ey.w, ey.y), fmaf(ox, ey.z, ey.x));
    f[2] = fmaf(ox, fmaf(oy, ez.w, ez.y), fmaf(oy, ez.z, ez.x));
    f[3] = fmaf(ox, bxy.y, bxy.x);
    f[4] = fmaf(oy, bxy.w, bxy.z);
    f[5] = fmaf(oz, bz.y, bz.x);
}

__device__ __forceinline__ void count_cross(DevCounters *ctr, int mask) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        unsigned b = __ballot_sync(0xffffffffu, (mask >> s) & 1);
        if (lane == 0 && b) atomicAdd(&ctr->cross[s], (unsigned long long)__popc(b));
    }
}

// Moves a particle by `shift` cells along one axis with the particle
// boundary of that axis; returns the crossed-side bits (bit 6: removed).
__device__ __forceinline__ int axis_bc(const BCTab &bc, int d, int n, int &i, float &o, float &u, float &v) {
    int mask = 0;
    if (i < 1) {  // left side: position (i - 1) + o < 0
        mask |= 1 << (2 * d);
        int kind = bc.pbc[2 * d];
        if (kind == PBC_PERIODIC) {
            i += n;
        } else if (kind == PBC_REFLECTING) {
            if (o == 0.0f) {
                i = 2 - i;
            } else {
                i = 1 - i;
                o = 1.0f - o;
            }
            u = -u;
            v = -v;
        } else {
            mask |= 1 << 6;
        }
    } else if (i > n) {  // right side: position > n
        mask |= 1 << (2 * d + 1);
        int kind = bc.pbc[2 * d + 1];
        if (kind == PBC_PERIODIC) {
            i -= n;
        } else if (kind == PBC_REFLECTING) {
            if (o == 0.0f) {
                i = 2 * n - i + 2;
            } else {
                i = 2 * n - i + 1;
                o = 1.0f - o;
            }
            u = -u;
            v = -v;
        } else {
            mask |= 1 << 6;
        }
    }
    return mask;
}

// The push of k_fused_m on one particle: Vay's pusher (REL) on u = gamma v,
// or Boris's; u is updated in place and v receives the new velocity. The
// adjoint kernel recomputes the step with this same function.
template <bool REL, bool FIRST>
__device__ __forceinline__ void push_m(const float f[6], const float qp, const float *g0, int64_t p, float &ux,
                                       float &uy, float &uz, float &vx, float &vy, float &vz) {
    if (REL) {
        // Vay's pusher (src/pusher/relativisticBoris.cpp:53-140) on
        // u = gamma v. Before the first push u holds the loaded v and
        // g0 the loaded gamma, which the reference multiplies in.
        float v0x, v0y, v0z, mx0, my0, mz0;
        if (FIRST) {
            v0x = ux; v0y = uy; v0z = uz;
            float g = g0[p];
            mx0 = g * ux; my0 = g * uy; mz0 = g * uz;
        } else {
            float iv = rsqrtf(1.0f + ux * ux + uy * uy + uz * uz);
            v0x = ux * iv; v0y = uy * iv; v0z = uz * iv;
            mx0 = ux; my0 = uy; mz0 = uz;
        }
        float vXbx = v0y * f[5] - v0z * f[4];
        float vXby = v0z * f[3] - v0x * f[5];
        float vXbz = v0x * f[4] - v0y * f[3];
        float upx = mx0 + qp * (f[0] + vXbx) + qp * f[0];
        float upy = my0 + qp * (f[1] + vXby) + qp * f[1];
        float upz = mz0 + qp * (f[2] + vXbz) + qp * f[2];
        float gps = 1.0f + upx * upx + upy * upy + upz * upz;
        float tx = qp * f[3], ty = qp * f[4], tz = qp * f[5];
        float tau2 = tx * tx + ty * ty + tz * tz;
        float sigma = gps - tau2;
        float ust = upx * tx + upy * ty + upz * tz;
        // sigma >= 1 (gps >= 1 + tau2), so both radicands are >= 1
        float rad = sigma * sigma + 4.0f * (tau2 + ust * ust);
        float igi = rsqrtf(0.5f * (sigma + rad * rsqrtf(rad)));
        tx *= igi;
        ty *= igi;
        tz *= igi;
        float sfac = __fdividef(1.0f, 1.0f + tx * tx + ty * ty + tz * tz);
        float ud = ust * igi;
        ux = sfac * (upx + ud * tx + (upy * tz - upz * ty));
        uy = sfac * (upy + ud * ty + (upz * tx - upx * tz));
        uz = sfac * (upz + ud * tz + (upx * ty - upy * tx));
        vx = ux * igi;
        vy = uy * igi;
        vz = uz * igi;
    } else {
        // Boris (src/pusher/boris.cpp:33-85)
        float tx = qp * f[3], ty = qp * f[4], tz = qp * f[5];
        float b2 = f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
        float ts = __fdividef(2.0f, 1.0f + qp * qp * b2);
        float sx = ts * tx, sy = ts * ty, sz = ts * tz;
        float mx = ux + qp * f[0], my = uy + qp * f[1], mz = uz + qp * f[2];
        float ix_ = mx + my * tz - mz * ty;
        float iy_ = my + mz * tx - mx * tz;
        float iz_ = mz + mx * ty - my * tx;
        ux = mx + iy_ * sz - iz_ * sy + qp * f[0];
        uy = my + iz_ * sx - ix_ * sz + qp * f[1];
        uz = mz + ix_ * sy - iy_ * sx + qp * f[2];
        vx = ux;
        vy = uy;
        vz = uz;
    }
}

constexpr int FUSED_BLOCK = 128;
constexpr int FUSED_WARPS = FUSED_BLOCK / 32;
constexpr int DEP_STRIDE = 33;  // column stride of the adjoint's transpose (odd: conflict-free both ways)
// Column stride of the fused kernel's deposit transpose: rows start on
// 16-byte boundaries, so a lane reads its 16 contributions of a row as four
// 16-byte loads; the column writes (a warp's 32 lanes, one row) stay
// conflict-free.
constexpr int COL_STRIDE = 36;

// One particle from FP64 position, velocity and gamma to the mixed state
// (cell, in-cell offsets, u); false when the position is outside the box or
// not a number. vmode (relativistic, before the first push): u holds v and
// g0 the loaded gamma. Shared by the loader and the host-resident step, so
// both convert bit-identically.
__device__ __forceinline__ bool f64_to_m(const Geom &g, const double pos[3], const double v[3], double ga, int rel,
                                         int vmode, int32_t &cell, float o[3], float u[3], float &g0) {
    int ci[3];
    bool ok = true;
    for (int d = 0; d < 3; d++) {
        double t = (pos[d] - g.x0[d]) * g.id[d];  // cells from x0
        double fl = floor(t);
        ci[d] = (int)fl + 1;
        float of = (float)(t - fl);
        if (of >= 1.0f) {
            of = 0.0f;
            ci[d] += 1;
        }
        o[d] = of;
        if (!(t == t) || ci[d] < 1 || ci[d] > g.n[d]) ok = false;
    }
    if (!ok) return false;
    cell = (int32_t)((int64_t)ci[0] * g.sx + (int64_t)ci[1] * g.sy + ci[2]);
    if (rel && vmode) {
        for (int d = 0; d < 3; d++) u[d] = (float)v[d];
        g0 = (float)ga;
    } else {
        const double f = rel ? ga : 1.0;
        for (int d = 0; d < 3; d++) u[d] = (float)(f * v[d]);
    }
    return true;
}

// The mixed state of one live particle back to FP64: out = x, y, z, vx, vy,
// vz, gamma (gamma 0 for the non-relativistic pusher, as new_particle()).
__device__ __forceinline__ void m_to_f64(const Geom &g, int32_t c, const float o[3], const float uf[3], int rel,
                                         double out[7]) {
    int ix = (int)(c / g.sx);
    int64_t r = c - ix * g.sx;
    int iy = (int)(r / g.sy);
    int iz = (int)(r - iy * g.sy);
    out[0] = g.x0[0] + g.d[0] * ((double)(ix - 1) + (double)o[0]);
    out[1] = g.x0[1] + g.d[1] * ((double)(iy - 1) + (double)o[1]);
    out[2] = g.x0[2] + g.d[2] * ((double)(iz - 1) + (double)o[2]);
    double ux = uf[0], uy = uf[1], uz = uf[2];
    double ga = rel ? sqrt(1.0 + ux * ux + uy * uy + uz * uz) : 1.0;
    out[3] = ux / ga;
    out[4] = uy / ga;
    out[5] = uz / ga;
    out[6] = rel ? ga : 0.0;
}

// A dropped particle in the caller's arrays, as the readback writes it.
__device__ __forceinline__ void host_dead(const MHost &H, int s, int64_t i) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    H.x[s][i] = H.y[s][i] = H.z[s][i] = H.vx[s][i] = H.vy[s][i] = H.vz[s][i] = nan;
    if (H.gam[s]) H.gam[s][i] = 0.0;
}

__device__ __forceinline__ void order2(float &a, float &b) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}

// A warp's list of J totals for cells other than the run reduction's (the
// corrected policy's pieces in a particle's old or intermediate cells), in
// shared memory, committed twelve lanes per entry, two entries per pass.
// Each total is rounded to the fixed-point quantum once and added with an
// integer atomic, so the order of the list does not change J.
constexpr int DEP_LIST = 32;

struct DepList {
    float (*val)[DEP_LIST + 1];  // [DEP_JSLOTS][DEP_LIST + 1]
    int *key;                    // [DEP_LIST]
    int n;                       // entries held (the same in every lane)
};

template <bool GUARD>
__device__ __forceinline__ void list_flush(DepList &L, const MDeposit &D, int lane) {
    __syncwarp();
    const int q = lane & 15, half = lane >> 4;
    if (q < DEP_JSLOTS) {
        const int pos = dep_pos(q);
        for (int e = half; e < L.n; e += 2)
            atomicAdd(D.wj + (size_t)L.key[e] * DEP_JSLOTS + pos, (unsigned long long)f2ll_rn<GUARD>(L.val[q][e]));
    }
    __syncwarp();
    L.n = 0;
}

// Appends (cell, v) of every lane with `has` set; called by all lanes.
template <bool GUARD>
__device__ __forceinline__ void list_append(DepList &L, const MDeposit &D, int lane, bool has, int cell,
                                            const float v[DEP_JSLOTS]) {
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (m == 0u) return;
    const int cnt = __popc(m);
    if (L.n + cnt > DEP_LIST) list_flush<GUARD>(L, D, lane);
    if (has) {
        const int e = L.n + __popc(m & lanemask_lt());
        L.key[e] = cell;
#pragma unroll
        for (int q = 0; q < DEP_JSLOTS; q++) L.val[q][e] = v[q];
    }
    L.n += cnt;
}

// Villasenor and Buneman's charge-conserving current of one particle's
// straight move (the corrected policy), the FP64 vb_deposit of
// particles_f64.cu in FP32 and in the old cell's units: s = the old in-cell
// offsets, e = s + the displacement in cells (|e - s| < 1 per axis). The path
// is split where it crosses a face (at most once per axis); the piece inside
// cell c (old cell + (-1, 0, 1) per axis, wrapped periodically) with extent D
// and mid-offsets m adds, for each axis a with transverse axes j, k, to its
// cell's slots 4a .. 4a+3
//   qd (D_a d_a / dt) ((1-m_j)(1-m_k) + D_j D_k/12, m_j (1-m_k) - .., m_j m_k + .., (1-m_j) m_k - ..).
// Pieces in the particle's new cell `onew` are summed into w (the run
// reduction commits them); the others are appended to the warp's list. All
// lanes of the warp call it (dep false: no pieces).
// Crossing times come from comparisons and one fast divide; the cell of a
// piece from comparisons (no conversion instruction).
// One straight piece of a path inside one cell, endpoints ua -> ub in the
// old cell's units (ix, iy, iz that cell): its cell's linear index (wrapped
// into [1, n] along periodic axes; a ghost cell along walled ones) and its
// twelve terms.
// The cell of the piece ua -> ub: its shift c (-1, 0, 1 per axis) from the
// mid-point and its linear index, wrapped into [1, n] along periodic axes, the
// ghost cell 0 or n + 1 along walled ones (mirrored back by the fold at a
// reflecting wall). Shared by the loop and its adjoint, so both place a piece
// alike.
__device__ __forceinline__ int vb_piece_cell(const MGeom &g, const int io[3], const float ua[3], const float ub[3],
                                             int c[3]) {
    int ct = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float mid = 0.5f * (ua[a] + ub[a]);
        c[a] = mid < 0.0f ? -1 : (mid >= 1.0f ? 1 : 0);
        int ii = io[a] + c[a];
        if (g.wrap[a]) ii = ii < 1 ? ii + g.n[a] : (ii > g.n[a] ? ii - g.n[a] : ii);
        ct += ii * (a == 0 ? (int)g.sx : a == 1 ? (int)g.sy : 1);
    }
    return ct;
}

__device__ __forceinline__ void vb_piece(const MGeom &g, const int io[3], const float ua[3], const float ub[3],
                                         float qd, int &ct, float W[DEP_JSLOTS]) {
    float m[3], Dd[3];
    int c[3];
    ct = vb_piece_cell(g, io, ua, ub, c);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float mid = 0.5f * (ua[a] + ub[a]);
        m[a] = mid - (c[a] < 0 ? -1.0f : (c[a] > 0 ? 1.0f : 0.0f));  // no int-to-float conversion (FP64 pipe)
        Dd[a] = ub[a] - ua[a];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int jb = (a + 1) % 3, kb = (a + 2) % 3;
        const float wa = qd * Dd[a] * g.ddt[a];
        const float cr = Dd[jb] * Dd[kb] * (1.0f / 12.0f);
        W[4 * a + 0] = wa * ((1.0f - m[jb]) * (1.0f - m[kb]) + cr);
        W[4 * a + 1] = wa * (m[jb] * (1.0f - m[kb]) - cr);
        W[4 * a + 2] = wa * (m[jb] * m[kb] + cr);
        W[4 * a + 3] = wa * ((1.0f - m[jb]) * m[kb] - cr);
    }
}

template <bool GUARD>
__device__ __forceinline__ void vb_pieces_list(const MGeom &g, const BCTab &bc, DepList &L, const MDeposit &D,
                                               int lane, bool dep, int ix, int iy, int iz, const float s[3],
                                               const float e[3], float qd, int onew, float w[DEP_JSLOTS]) {
    float t[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool lo = e[a] < 0.0f, hi = e[a] >= 1.0f;
        t[a] = (lo || hi) ? __fdividef((hi ? 1.0f : 0.0f) - s[a], e[a] - s[a]) : 2.0f;
    }
    order2(t[0], t[1]);
    order2(t[1], t[2]);
    order2(t[0], t[1]);
    const int io[3] = {ix, iy, iz};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float ta = k == 0 ? 0.0f : fminf(t[k - 1], 1.0f);
        const float tb = k == 3 ? 1.0f : fminf(t[k], 1.0f);
        const bool valid = dep && tb > ta;
        float W[DEP_JSLOTS];
        int ct = 0;
        if (valid) {
            float ua[3], ub[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float de = e[a] - s[a];
                ua[a] = fmaf(ta, de, s[a]);
                ub[a] = fmaf(tb, de, s[a]);
            }
            vb_piece(g, io, ua, ub, qd, ct, W);
            if (ct == onew) {
#pragma unroll
                for (int q = 0; q < DEP_JSLOTS; q++) w[q] += W[q];
            }
        }
        list_append<GUARD>(L, D, lane, valid && ct != onew, ct, W);
    }
    // a move that ends beyond an absorbing wall removes the particle: its path
    // continues along the wall's normal to the next vertex plane beyond the
    // wall (offset -1 or 2 in the old cell's units), so that its whole charge
    // crosses the wall's plane (the FP64 form's absorbed_exit)
    const bool absorbs = bc.pbc[0] == PBC_ABSORBING || bc.pbc[1] == PBC_ABSORBING || bc.pbc[2] == PBC_ABSORBING ||
                         bc.pbc[3] == PBC_ABSORBING || bc.pbc[4] == PBC_ABSORBING || bc.pbc[5] == PBC_ABSORBING;
    if (!absorbs) return;  // the same for every lane
    float a0[3] = {e[0], e[1], e[2]};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int io_a = a == 0 ? ix : a == 1 ? iy : iz;
        const bool left = bc.pbc[2 * a] == PBC_ABSORBING && io_a == 1 && a0[a] < 0.0f;
        const bool right = bc.pbc[2 * a + 1] == PBC_ABSORBING && io_a == g.n[a] && a0[a] >= 1.0f;
        const bool has = dep && (left || right);
        float W[DEP_JSLOTS];
        int ct = 0;
        if (has) {
            float b0[3] = {a0[0], a0[1], a0[2]};
            b0[a] = left ? -1.0f : 2.0f;
            vb_piece(g, io, a0, b0, qd, ct, W);
            a0[a] = b0[a];
        }
        list_append<GUARD>(L, D, lane, has, ct, W);
    }
}

// Fused gather + push + boundaries + deposit, one thread per particle.
//
// Deposit: each lane writes its particle's 20 contributions as a column of a
// per-warp 20 x 32 shared array; then lane q walks row q, summing the
// contributions of each run of consecutive particles that share a cell in
// particle order, and adds each run total, in int64 fixed point, to slot q of
// the run's cell. The order of every FP32 sum is fixed by the particle order,
// so the slots are bit-reproducible. A warp whose particles are all in
// different cells (before the first sort) commits each particle directly.
//
// Division and square roots use the hardware approximations (rsqrtf,
// __fdividef, relative error a few 2^-24): the form's accuracy is FP32. No
// conversion instruction runs per particle (see f2ll_rn, cell_step).
//
// CORR: the corrected policy - the pack holds true-vertex coefficients, the
// deposit at the current state uses the weights 1 - o and o, and the time
// loop's current is the charge-conserving one of vb_pieces_list.
//
// HOST (with PUSH, after the first push): the particle state is read from and
// written back to the caller's FP64 arrays (Hp) instead of the device store,
// converted as the loader and readback convert (f64_to_m, m_to_f64), so one
// launch moves every particle over the host link in both directions at once.
// Resident blocks per SM the register budget is cut for, counted in blocks of
// 256 threads and measured over a 20-step sort interval at 256^3: 6 (40
// registers, no spills) for the reference policy on the device store, where
// more warps hide the L2 latency that grows as particles drift between sorts
// (12.59 against 13.06 ms a launch at 5); 4 (64 registers, no spills) for the
// corrected policy's pieces (19.23 against 20.01 ms at 5 with 148 bytes of
// spills, 24.6 ms at 6); 5 (48 registers) for the host-resident conversions.
// The same warps in blocks of 128 threads, twice as many blocks, take 12.36
// ms (blocks of 64: 12.60; of 96: 12.63; of 512: 12.92).
template <bool CORR, bool HOST>
constexpr int fused_min_blocks() {
    return 256 / FUSED_BLOCK * (CORR ? 4 : (HOST ? 5 : 6));
}

template <bool REL, bool FIRST, bool PUSH, bool CORR = false, bool HOST = false>
__global__ void __launch_bounds__(FUSED_BLOCK, fused_min_blocks<CORR, HOST>())
    k_fused_m(MGeom g, Div3 dv, MSpecies st, BCTab bc, const float4 *__restrict__ pack, MState S, int64_t np,
              MDeposit D, int with_rho, const float *g0, DevCounters *ctr, const MHost *__restrict__ Hp,
              int store_pre) {
    __shared__ __align__(16) float s_w[FUSED_WARPS][20 * COL_STRIDE];
    __shared__ int s_key[FUSED_WARPS][32];
    constexpr bool VBL = CORR && PUSH;  // the corrected policy's pieces go through a list
    __shared__ float s_pl[VBL ? FUSED_WARPS : 1][DEP_JSLOTS][DEP_LIST + 1];
    __shared__ int s_plk[VBL ? FUSED_WARPS : 1][DEP_LIST];
    // a 32-bit product (mixed_fused refuses 2^32 particles or more): the state
    // arrays are then addressed with one wide multiply-add each
    const int64_t p = (int64_t)(blockIdx.x * blockDim.x + threadIdx.x);
    const int lane = threadIdx.x & 31;
    float *col = s_w[threadIdx.x >> 5];
    int *keys = s_key[threadIdx.x >> 5];
    bool active = false;
    int mask = 0;
    int onew = 0;
    // the corrected policy's move, for its pieces after the divergent part
    bool vb_dep = false;
    int vb_i[3] = {0, 0, 0};
    float vb_s[3] = {0.0f, 0.0f, 0.0f}, vb_e[3] = {0.0f, 0.0f, 0.0f}, vb_qd = 0.0f;
    if (p < np) {
        int32_t c;
        float ox, oy, oz, ux, uy, uz;
        int hs = 0;
        int64_t hi = 0;
        if (HOST) {
            hs = species_of_m(st, p);
            hi = p - st.off[hs];
            const double pos[3] = {Hp->x[hs][hi], Hp->y[hs][hi], Hp->z[hs][hi]};
            const double v[3] = {Hp->vx[hs][hi], Hp->vy[hs][hi], Hp->vz[hs][hi]};
            const double ga = Hp->gam[hs] ? Hp->gam[hs][hi] : 0.0;
            float o3[3], u3[3], gz;
            if (f64_to_m(Hp->g, pos, v, ga, Hp->rel, 0, c, o3, u3, gz)) {
                ox = o3[0], oy = o3[1], oz = o3[2];
                ux = u3[0], uy = u3[1], uz = u3[2];
            } else {  // outside the box (the loader's bounds check): dropped as the readback drops it
                if (pos[0] == pos[0]) atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
                host_dead(*Hp, hs, hi);
                c = -1;
            }
            if (store_pre) {  // the state before the push into the device store, as an upload leaves it
                S.cell[p] = c;
                if (c >= 0) {
                    S.ox[p] = ox, S.oy[p] = oy, S.oz[p] = oz;
                    S.ux[p] = ux, S.uy[p] = uy, S.uz[p] = uz;
                }
            }
        } else {
            c = S.cell[p];
        }
        if (c >= 0) {
            const int s = species_of_m(st, p);
            if (!HOST) {
                ox = S.ox[p], oy = S.oy[p], oz = S.oz[p];
                ux = S.ux[p], uy = S.uy[p], uz = S.uz[p];
            }
            float vx, vy, vz;
            int ix, iy, iz;
            split_cell(g, dv, c, ix, iy, iz);
            const int ix0 = ix, iy0 = iy, iz0 = iz;
            const float so[3] = {ox, oy, oz};
            float mv[3] = {0.0f, 0.0f, 0.0f};
            if (!PUSH) {
                // deposit at the current state (Particle_Handler::depositRhoJ)
                float iga = 1.0f;
                if (REL && !FIRST) iga = rsqrtf(1.0f + ux * ux + uy * uy + uz * uz);
                vx = ux * iga;
                vy = uy * iga;
                vz = uz * iga;
            } else {
                float f[6];
                gather_pack(pack + (int64_t)c * PACK_F4, ox, oy, oz, f);
                push_m<REL, FIRST>(f, st.qp[s], g0, p, ux, uy, uz, vx, vy, vz);
                // position update in cell units, then the boundaries per axis
                float nx = ox + vx * g.dtid[0], ny = oy + vy * g.dtid[1], nz = oz + vz * g.dtid[2];
                mv[0] = nx;
                mv[1] = ny;
                mv[2] = nz;
                cell_step(nx, ix, ox);
                cell_step(ny, iy, oy);
                cell_step(nz, iz, oz);
                mask |= axis_bc(bc, 0, g.n[0], ix, ox, ux, vx);
                if (!(mask & 64)) mask |= axis_bc(bc, 1, g.n[1], iy, oy, uy, vy);
                if (!(mask & 64)) mask |= axis_bc(bc, 2, g.n[2], iz, oz, uz, vz);
            }
            if (VBL && (mask & 64) && st.deposit[s]) {
                // an absorbing wall removed the particle: the current of its
                // whole move still goes in (pieces after the branch)
                vb_dep = true;
                vb_i[0] = ix0, vb_i[1] = iy0, vb_i[2] = iz0;
#pragma unroll
                for (int a = 0; a < 3; a++) vb_s[a] = so[a], vb_e[a] = mv[a];
                vb_qd = st.qdep[s];
            }
            if (mask & 64) {
                if (HOST) host_dead(*Hp, hs, hi);
                else S.cell[p] = -1;
            } else if (ix < 1 || ix > g.n[0] || iy < 1 || iy > g.n[1] || iz < 1 || iz > g.n[2]) {
                // moved more than a box length in one step: record, drop
                atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
                if (HOST) host_dead(*Hp, hs, hi);
                else S.cell[p] = -1;
                mask |= 64;
            } else {
                onew = ix * (int)g.sx + iy * (int)g.sy + iz;  // < npts < 2^31 (checked in mixed_alloc)
                if (PUSH && HOST) {
                    const float o3[3] = {ox, oy, oz}, u3[3] = {ux, uy, uz};
                    double out[7];
                    m_to_f64(Hp->g, onew, o3, u3, Hp->rel, out);
                    Hp->x[hs][hi] = out[0];
                    Hp->y[hs][hi] = out[1];
                    Hp->z[hs][hi] = out[2];
                    Hp->vx[hs][hi] = out[3];
                    Hp->vy[hs][hi] = out[4];
                    Hp->vz[hs][hi] = out[5];
                    if (Hp->gam[hs]) Hp->gam[hs][hi] = out[6];
                } else if (PUSH) {
                    S.cell[p] = onew;
                    S.ox[p] = ox;
                    S.oy[p] = oy;
                    S.oz[p] = oz;
                    S.ux[p] = ux;
                    S.uy[p] = uy;
                    S.uz[p] = uz;
                }
                if (CORR && PUSH && st.deposit[s]) {
                    active = true;
                    vb_dep = true;
                    vb_i[0] = ix0, vb_i[1] = iy0, vb_i[2] = iz0;
#pragma unroll
                    for (int a = 0; a < 3; a++) vb_s[a] = so[a], vb_e[a] = mv[a];
                    vb_qd = st.qdep[s];
                    float *w = col + lane;
                    if (with_rho) {  // rho at the new position, true-vertex weights
                        const float qd = st.qdep[s];
                        const float a[3] = {1.0f - ox, 1.0f - oy, 1.0f - oz}, b[3] = {ox, oy, oz};
                        w[12 * COL_STRIDE] = qd * a[0] * a[1] * a[2];
                        w[13 * COL_STRIDE] = qd * b[0] * a[1] * a[2];
                        w[14 * COL_STRIDE] = qd * b[0] * b[1] * a[2];
                        w[15 * COL_STRIDE] = qd * a[0] * b[1] * a[2];
                        w[16 * COL_STRIDE] = qd * a[0] * b[1] * b[2];
                        w[17 * COL_STRIDE] = qd * b[0] * b[1] * b[2];
                        w[18 * COL_STRIDE] = qd * b[0] * a[1] * b[2];
                        w[19 * COL_STRIDE] = qd * a[0] * a[1] * b[2];
                    }
                } else if (st.deposit[s]) {
                    active = true;
                    // deposit weights (src/particles/deposit.cpp:12-62) in
                    // fixed-point units: (UNIT_RHOJ q / V) v_i (2 - o_j)(2 - o_k) etc.;
                    // over the true vertex (CORR) 1 - o and o
                    float a[3] = {2.0f - ox, 2.0f - oy, 2.0f - oz};
                    float b[3] = {ox - 1.0f, oy - 1.0f, oz - 1.0f};
                    if (CORR) {
                        a[0] = 1.0f - ox, a[1] = 1.0f - oy, a[2] = 1.0f - oz;
                        b[0] = ox, b[1] = oy, b[2] = oz;
                    }
                    const float qd = st.qdep[s];
                    float jx = qd * vx, jy = qd * vy, jz = qd * vz;
                    float *w = col + lane;
                    w[0 * COL_STRIDE] = jx * a[1] * a[2];
                    w[1 * COL_STRIDE] = jx * b[1] * a[2];
                    w[2 * COL_STRIDE] = jx * b[1] * b[2];
                    w[3 * COL_STRIDE] = jx * a[1] * b[2];
                    w[4 * COL_STRIDE] = jy * a[2] * a[0];
                    w[5 * COL_STRIDE] = jy * b[2] * a[0];
                    w[6 * COL_STRIDE] = jy * b[2] * b[0];
                    w[7 * COL_STRIDE] = jy * a[2] * b[0];
                    w[8 * COL_STRIDE] = jz * a[0] * a[1];
                    w[9 * COL_STRIDE] = jz * b[0] * a[1];
                    w[10 * COL_STRIDE] = jz * b[0] * b[1];
                    w[11 * COL_STRIDE] = jz * a[0] * b[1];
                    if (with_rho) {
                        w[12 * COL_STRIDE] = qd * a[0] * a[1] * a[2];
                        w[13 * COL_STRIDE] = qd * b[0] * a[1] * a[2];
                        w[14 * COL_STRIDE] = qd * b[0] * b[1] * a[2];
                        w[15 * COL_STRIDE] = qd * a[0] * b[1] * a[2];
                        w[16 * COL_STRIDE] = qd * a[0] * b[1] * b[2];
                        w[17 * COL_STRIDE] = qd * b[0] * b[1] * b[2];
                        w[18 * COL_STRIDE] = qd * b[0] * a[1] * b[2];
                        w[19 * COL_STRIDE] = qd * a[0] * a[1] * b[2];
                    }
                }
            }
        }
    }
    if (VBL) {
        // Villasenor-Buneman pieces with the whole warp present: the new
        // cell's into the column, the others through the warp's list
        DepList PL{s_pl[threadIdx.x >> 5], s_plk[threadIdx.x >> 5], 0};
        float wv[DEP_JSLOTS];
#pragma unroll
        for (int q = 0; q < DEP_JSLOTS; q++) wv[q] = 0.0f;
        // a particle the boundaries removed has no new cell: all its pieces go to the list
        vb_pieces_list<true>(g, bc, PL, D, lane, vb_dep, vb_i[0], vb_i[1], vb_i[2], vb_s, vb_e, vb_qd,
                             active ? onew : -1, wv);
        if (PL.n) list_flush<true>(PL, D, lane);
        if (vb_dep && active) {
#pragma unroll
            for (int q = 0; q < DEP_JSLOTS; q++) col[q * COL_STRIDE + lane] = wv[q];
        }
    }
    if (__any_sync(0xffffffffu, mask & 63)) count_cross(ctr, mask & 63);
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (act == 0u) return;
    // runs of equal cells (inactive lanes get unique negative keys)
    const int key = active ? onew : -1 - lane;
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != key);
    keys[lane] = active ? onew : -1;
    if (!active) {
#pragma unroll
        for (int q = 0; q < DEP_SLOTS; q++) col[q * COL_STRIDE + lane] = 0.0f;
    }
    __syncwarp();
    const int nq = with_rho ? DEP_SLOTS : 12;
    if (heads == 0xffffffffu) {
        // every particle in a cell of its own (unsorted input)
        if (active) {
            unsigned long long *dj = D.wj + (size_t)onew * DEP_JSLOTS, *dr = D.wr + (size_t)onew * DEP_RSLOTS;
#pragma unroll
            for (int q = 0; q < DEP_SLOTS; q++) {
                if (q >= nq) break;
                long long fx = f2ll_rn(col[q * COL_STRIDE + lane]);
                if (fx != 0) atomicAdd((q < 12 ? dj : dr) + dep_pos(q), (unsigned long long)fx);
            }
        }
        return;
    }
    const unsigned ends32 = (heads >> 1) | 0x80000000u;  // bit i: particle i ends its run
    if (nq == DEP_JSLOTS) {
        // J only (the time loop): lanes 0..11 walk rows 0..11 over particles
        // 0..15 while lanes 16..27 walk them over particles 16..31, each in
        // particle order, committing at each run end; a run that spans
        // particles 15 and 16 is committed as two parts.
        // Only the ends of active runs commit: an inactive particle is a run of
        // its own with a zero column, so skipping its end adds 0 to the next run.
        // With |velocity| < 1 (relativistic), a run total is below 2^39 quanta.
        const int q = lane & 15, half = lane >> 4;
        if (q < DEP_JSLOTS) {
            unsigned long long *dst = D.wj + dep_pos(q);
            const float4 *row = reinterpret_cast<const float4 *>(col + q * COL_STRIDE + 16 * half);
            const int *hkeys = keys + 16 * half;
            const unsigned hact = (act >> (16 * half)) & 0xffffu;
            const unsigned ends = (((ends32 >> (16 * half)) & 0xffffu) | 0x8000u) & hact;
            float r[16];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float4 v = row[i];
                r[4 * i] = v.x, r[4 * i + 1] = v.y, r[4 * i + 2] = v.z, r[4 * i + 3] = v.w;
            }
            float acc = 0.0f;
#pragma unroll
            for (int i = 0; i < 16; i++) {
                acc += r[i];
                if ((ends >> i) & 1u) {
                    atomicAdd(dst + (size_t)hkeys[i] * DEP_JSLOTS, (unsigned long long)f2ll_rn<!REL>(acc));
                    acc = 0.0f;
                }
            }
        }
        return;
    }
    if (lane < nq) {
        // row `lane`: one pass in particle order, committing at each run end;
        // lanes 0..11 commit one cell's J record together, lanes 12..19 its rho record
        const bool jrow = lane < 12;
        unsigned long long *dst = (jrow ? D.wj : D.wr) + dep_pos(lane);
        const int stride = jrow ? DEP_JSLOTS : DEP_RSLOTS;
        const float4 *row = reinterpret_cast<const float4 *>(col + lane * COL_STRIDE);
        const unsigned ends = ends32;
        float acc = 0.0f;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float r[16];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float4 v = row[4 * h + i];
                r[4 * i] = v.x, r[4 * i + 1] = v.y, r[4 * i + 2] = v.z, r[4 * i + 3] = v.w;
            }
#pragma unroll
            for (int i = 0; i < 16; i++) {
                acc += r[i];
                if ((ends >> (16 * h + i)) & 1u) {  // warp-uniform
                    const int kk = keys[16 * h + i];
                    if (kk >= 0) {
                        // zero totals are committed too: testing costs more than the atomic
                        atomicAdd(dst + (size_t)kk * stride, (unsigned long long)f2ll_rn(acc));
                    }
                    acc = 0.0f;
                }
            }
        }
    }
}

// J (what & 1) and rho (what & 2) at every grid point from the per-cell
// records: point p gathers slot q of cell p - off(q), the inverse of the
// deposit table. Integer sums, so the result equals committing every run
// total to its point directly.
//
// corr: the corrected policy's Jx index - slot 4 (q 3) feeds point cell + 1,
// not cell + sy (src/grid/oGrid.cpp:101 as the reference has it).
__global__ void k_cells_to_points(int64_t npts, int sx, int sy, const unsigned long long *__restrict__ wj,
                                  const unsigned long long *__restrict__ wr, unsigned long long *Jx,
                                  unsigned long long *Jy, unsigned long long *Jz, unsigned long long *rho, int what,
                                  int corr) {
    // points from sx + sy + 1 on have every neighbour record; below that (the
    // low ghost planes, which only walled dimensions' pieces reach) each
    // record is read where it exists
    const int64_t first = (int64_t)sx + sy + 1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts; p += (int64_t)gridDim.x * blockDim.x) {
        if (p < first) {
            auto slot = [&](const unsigned long long *w, int ns, int64_t c, int k) -> unsigned long long {
                return c >= 0 ? w[c * ns + k] : 0ull;
            };
            if (what & 1) {
                const unsigned long long q3 = corr ? slot(wj, DEP_JSLOTS, p - 1, 4) : slot(wj, DEP_JSLOTS, p - sy, 4);
                Jx[p] = slot(wj, DEP_JSLOTS, p, 0) + slot(wj, DEP_JSLOTS, p - sy, 3) + q3 +
                        slot(wj, DEP_JSLOTS, p - sy - 1, 7);
                Jy[p] = slot(wj, DEP_JSLOTS, p, 1) + slot(wj, DEP_JSLOTS, p - 1, 6) +
                        slot(wj, DEP_JSLOTS, p - sx - 1, 8) + slot(wj, DEP_JSLOTS, p - sx, 10);
                Jz[p] = slot(wj, DEP_JSLOTS, p, 2) + slot(wj, DEP_JSLOTS, p - sy, 5) +
                        slot(wj, DEP_JSLOTS, p - sx - sy, 9) + slot(wj, DEP_JSLOTS, p - sx, 11);
            }
            if (what & 2)
                rho[p] = slot(wr, DEP_RSLOTS, p, 0) + slot(wr, DEP_RSLOTS, p - sy, 1) + slot(wr, DEP_RSLOTS, p - 1, 2) +
                         slot(wr, DEP_RSLOTS, p - sy - 1, 3) + slot(wr, DEP_RSLOTS, p - sx - 1, 4) +
                         slot(wr, DEP_RSLOTS, p - sx - sy, 5) + slot(wr, DEP_RSLOTS, p - sx, 6) +
                         slot(wr, DEP_RSLOTS, p - sx - sy - 1, 7);
            continue;
        }
        if (what & 1) {
            unsigned long long jx = 0, jy = 0, jz = 0;
            {
                // J record of cell c: wj + 12 c (96 bytes, 32-byte aligned)
                auto rec = [&](int64_t c) { return wj + c * DEP_JSLOTS; };
                const ulonglong2 g0a = __ldg(reinterpret_cast<const ulonglong2 *>(rec(p)));        // slots 0,1
                const unsigned long long g0b = __ldg(rec(p) + 2);
                const unsigned long long g2a = __ldg(rec(p - sy) + 3);
                const ulonglong2 g2b = __ldg(reinterpret_cast<const ulonglong2 *>(rec(p - sy) + 4));  // 4,5
                const unsigned long long g1 = __ldg(rec(p - 1) + 6);
                const unsigned long long g3 = __ldg(rec(p - sy - 1) + 7);
                const unsigned long long g5 = __ldg(rec(p - sx - 1) + 8);
                const unsigned long long g6 = __ldg(rec(p - sx - sy) + 9);
                const ulonglong2 g4 = __ldg(reinterpret_cast<const ulonglong2 *>(rec(p - sx) + 10));  // 10,11
                const unsigned long long q3 = corr ? __ldg(rec(p - 1) + 4) : g2b.x;
                jx = g0a.x + g2a + q3 + g3;      // q 0, 1, 3, 2
                jy = g0a.y + g1 + g5 + g4.x;     // q 4, 5, 6, 7
                jz = g0b + g2b.y + g6 + g4.y;    // q 8, 11, 10, 9
            }
            Jx[p] = jx;
            Jy[p] = jy;
            Jz[p] = jz;
        }
        if (what & 2) {
            unsigned long long r = 0;
            {
                auto rec = [&](int64_t c) { return wr + c * DEP_RSLOTS; };
                r = __ldg(rec(p)) + __ldg(rec(p - sy) + 1) + __ldg(rec(p - 1) + 2) + __ldg(rec(p - sy - 1) + 3) +
                    __ldg(rec(p - sx - 1) + 4) + __ldg(rec(p - sx - sy) + 5) + __ldg(rec(p - sx) + 6) +
                    __ldg(rec(p - sx - sy - 1) + 7);  // q 12 15 19 16 18 14 13 17
            }
            rho[p] = r;
        }
    }
}

// ---- conversions --------------------------------------------------------

// vmode (relativistic, before the first push): the momentum slots take the
// loaded velocity and g0 the loaded gamma; otherwise u = gamma v directly.
__global__ void k_from_f64(Geom g, MState S, int64_t at, int64_t n, const double *x, const double *y,
                           const double *z, const double *vx, const double *vy, const double *vz, const double *gam,
                           int rel, int vmode, float *g0, DevCounters *ctr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double pos[3] = {x[i], y[i], z[i]}, v[3] = {vx[i], vy[i], vz[i]};
        const double ga = gam ? gam[i] : 0.0;  // new_particle() leaves gamma at 0
        int32_t cell;
        float o[3], u[3], gz = 0.0f;
        const int64_t p = at + i;
        if (!f64_to_m(g, pos, v, ga, rel, vmode, cell, o, u, gz)) {
            atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
            S.cell[p] = -1;
            continue;
        }
        S.cell[p] = cell;
        S.ox[p] = o[0];
        S.oy[p] = o[1];
        S.oz[p] = o[2];
        S.ux[p] = u[0];
        S.uy[p] = u[1];
        S.uz[p] = u[2];
        if (rel && vmode) g0[p] = gz;
    }
}

__global__ void k_to_f64(Geom g, MState S, int64_t at, int64_t n, double *x, double *y, double *z, double *vx,
                         double *vy, double *vz, double *gam, int rel, const float *g0) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = at + i;
        int32_t c = S.cell[p];
        if (c < 0) {
            x[i] = y[i] = z[i] = vx[i] = vy[i] = vz[i] = __longlong_as_double(0x7ff8000000000000LL);
            if (gam) gam[i] = 0.0;
            continue;
        }
        const float o[3] = {S.ox[p], S.oy[p], S.oz[p]}, u[3] = {S.ux[p], S.uy[p], S.uz[p]};
        double out[7];
        m_to_f64(g, c, o, u, rel, out);
        x[i] = out[0];
        y[i] = out[1];
        z[i] = out[2];
        if (rel && g0) {  // before the first push: loaded v and gamma
            vx[i] = u[0];
            vy[i] = u[1];
            vz[i] = u[2];
            if (gam) gam[i] = (double)g0[p];
            continue;
        }
        vx[i] = out[3];
        vy[i] = out[4];
        vz[i] = out[5];
        if (gam) gam[i] = out[6];
    }
}

__global__ void k_d2f(const double *a, float *b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void k_f2d(const float *a, double *b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}
__global__ void k_fix2d(const long long *a, double *b, int64_t n, double q0) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i] * q0;
}
__global__ void k_d2fix(const double *a, long long *b, int64_t n, double iq0) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __double2ll_rn(a[i] * iq0);
}
__global__ void k_fillf(float *a, int64_t n, float v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

// ---- FP32 grid kernels ---------------------------------------------------

struct MF3 {
    float *p[3];
};
struct MCF3 {
    const float *p[3];
};
struct MJ3 {
    const long long *p[3];
};

__global__ void k_yee_e_m(MGeom g, MF3 E, MCF3 T, MJ3 J, float dt, float q0) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = (int64_t)i * g.sx + (int64_t)j * g.sy + k;
    const float *Tx = T.p[0], *Ty = T.p[1], *Tz = T.p[2];
    float jx = __ll2float_rn(J.p[0][o]) * q0, jy = __ll2float_rn(J.p[1][o]) * q0, jz = __ll2float_rn(J.p[2][o]) * q0;
    E.p[0][o] -= dt * ((Ty[o] - Ty[o - 1]) * g.idf[2] - (Tz[o] - Tz[o - g.sy]) * g.idf[1] + FOURPI_F * jx);
    E.p[1][o] -= dt * ((Tz[o] - Tz[o - g.sx]) * g.idf[0] - (Tx[o] - Tx[o - 1]) * g.idf[2] + FOURPI_F * jy);
    E.p[2][o] -= dt * ((Tx[o] - Tx[o - g.sy]) * g.idf[1] - (Ty[o] - Ty[o - g.sx]) * g.idf[0] + FOURPI_F * jz);
}

__global__ void k_yee_b_m(MGeom g, MF3 B, MCF3 T, MCF3 E, float dt) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = (int64_t)i * g.sx + (int64_t)j * g.sy + k;
    const float *Ex = E.p[0], *Ey = E.p[1], *Ez = E.p[2];
    B.p[0][o] = T.p[0][o] + dt * ((Ey[o + 1] - Ey[o]) * g.idf[2] - (Ez[o + g.sy] - Ez[o]) * g.idf[1]);
    B.p[1][o] = T.p[1][o] + dt * ((Ez[o + g.sx] - Ez[o]) * g.idf[0] - (Ex[o + 1] - Ex[o]) * g.idf[2]);
    B.p[2][o] = T.p[2][o] + dt * ((Ex[o + g.sy] - Ex[o]) * g.idf[1] - (Ey[o + g.sx] - Ey[o]) * g.idf[0]);
}

__global__ void k_yee_es_m(MGeom g, MF3 E, MJ3 J, float dt, float q0) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = (int64_t)i * g.sx + (int64_t)j * g.sy + k;
    for (int c = 0; c < 3; c++) E.p[c][o] = -dt * (FOURPI_F * (__ll2float_rn(J.p[c][o]) * q0));
}

struct MList6 {
    float *p[6];
    int n;
};

// Periodic ghost fill over the physical transverse range (same scheme as the
// FP64 k_ghost): all copies read physical points, any dims run at once.
__global__ void k_ghost_m(MGeom g, MList6 fl, int dims_mask) {
    int z = blockIdx.z;
    int r = z & 1;
    int d = (z >> 1) % 3;
    int f = (z >> 1) / 3;
    if (!((dims_mask >> d) & 1) || f >= fl.n) return;
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int p = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || p > g.n[o1]) return;
    int nd = g.n[d];
    int src = r == 0 ? nd : 1, dst = r == 0 ? 0 : nd + 1;
    int is[3], it[3];
    is[d] = src;
    it[d] = dst;
    is[o1] = it[o1] = p;
    is[o2] = it[o2] = q;
    float *F = fl.p[f];
    F[(int64_t)it[0] * g.sx + (int64_t)it[1] * g.sy + it[2]] = F[(int64_t)is[0] * g.sx + (int64_t)is[1] * g.sy + is[2]];
}

// Periodic fold of one dimension on the fixed-point accumulators (exact
// integer adds); the folded ghost plane is left as the reference leaves it.
__global__ void k_fold_m(MGeom g, int d, long long *f0, long long *f1, long long *f2) {
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int p = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || p > g.n[o1]) return;
    int is[3], it[3];
    is[d] = g.n[d] + 1;
    it[d] = 1;
    is[o1] = it[o1] = p;
    is[o2] = it[o2] = q;
    int64_t s = (int64_t)is[0] * g.sx + (int64_t)is[1] * g.sy + is[2];
    int64_t t = (int64_t)it[0] * g.sx + (int64_t)it[1] * g.sy + it[2];
    long long *F = blockIdx.z == 0 ? f0 : (blockIdx.z == 1 ? f1 : f2);
    F[t] += F[s];
}

// The corrected policy's periodic fold and ghost fill along dim d over the
// whole (n+3)^2 plane (dimension by dimension, so edge and corner lines
// follow), as k_periodic_full of the FP64 form: fold f[n] += f[0],
// f[1] += f[n+1], f[2] += f[n+2] (exact integer adds) on the fixed-point
// arrays; ghost f[0] = f[n], f[n+1] = f[1], f[n+2] = f[2] on the FP32 ones.
// One array per blockIdx.z.
struct MFix4 {
    long long *p[4];
};
struct MF9 {
    float *p[9];
};

template <class T>
__device__ __forceinline__ void periodic_full_line(const MGeom &g, T *F, int d, int r, int q, bool fold) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int n = g.n[d];
    int c[3];
    c[o1] = r;
    c[o2] = q;
    auto at = [&](int i) -> T & {
        c[d] = i;
        return F[(int64_t)c[0] * g.sx + (int64_t)c[1] * g.sy + c[2]];
    };
    if (fold) {
        at(n) += at(0);
        at(1) += at(n + 1);
        at(2) += at(n + 2);
    } else {
        at(0) = at(n);
        at(n + 1) = at(1);
        at(n + 2) = at(2);
    }
}

__global__ void k_fold_full_m(MGeom g, MFix4 fl, int d, int t1, int t2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= t2 || r >= t1) return;
    periodic_full_line(g, fl.p[blockIdx.z], d, r, q, true);
}

__global__ void k_ghost_full_m(MGeom g, MF9 fl, int d, int t1, int t2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= t2 || r >= t1) return;
    periodic_full_line(g, fl.p[blockIdx.z], d, r, q, false);
}

struct MPlane {
    float *f;
    int dim, idx;
    float v, vs;
    const float *t1, *t2;  // transverse spot factors, or null (PlaneSet)
};
struct MPlaneList {
    MPlane s[12];
    int n;
};

__global__ void k_plane_m(MGeom g, MPlaneList pl, int tot0, int tot1, int tot2) {
    int e = blockIdx.z;
    if (e >= pl.n) return;
    const MPlane &ps = pl.s[e];
    int d = ps.dim;
    int tot[3] = {tot0, tot1, tot2};
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int p = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= tot[o2] || p >= tot[o1]) return;
    int ii[3];
    ii[d] = ps.idx;
    ii[o1] = p;
    ii[o2] = q;
    float v = ps.v;
    if (ps.t1) v += ps.vs * ps.t1[p] * ps.t2[q];
    ps.f[(int64_t)ii[0] * g.sx + (int64_t)ii[1] * g.sy + ii[2]] = v;
}

// ---- reductions (FP64 accumulation) -------------------------------------

// The history reductions take their per-particle (per-cell) terms in FP32,
// sum them in FP32 over at most DIAG_CHUNK items per thread and accumulate
// those partial sums in FP64: FP64 arithmetic per item would run on the
// narrow FP64 pipe (2 lanes per clock per SM on this GPU), which made these
// reductions cost more than a whole step. The partition is fixed by the launch
// shape, so the sums are reproducible.
constexpr int DIAG_CHUNK = 8;

__global__ void k_moments_m(MSpecies st, MState S, int64_t np, int rel, const float *g0, double *part) {
    double acc[4] = {0, 0, 0, 0};
    float f[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int k = 0;
    const bool gam = rel && !g0;  // before the first push u holds v
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        if (S.cell[p] >= 0) {
            const float ux = S.ux[p], uy = S.uy[p], uz = S.uz[p];
            const float iv = gam ? 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz) : 1.0f;
            const float vx = ux * iv, vy = uy * iv, vz = uz * iv;
            const float m = st.m[species_of_m(st, p)];
            f[0] += 0.5f * m * (vx * vx + vy * vy + vz * vz);
            f[1] += m * vx;
            f[2] += m * vy;
            f[3] += m * vz;
        }
        if (++k == DIAG_CHUNK) {
            for (int q = 0; q < 4; q++) {
                acc[q] += (double)f[q];
                f[q] = 0.0f;
            }
            k = 0;
        }
    }
    for (int q = 0; q < 4; q++) acc[q] += (double)f[q];
    __shared__ double sh[32][4];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 4; q++) {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) v += sh[ww][threadIdx.x];
        part[blockIdx.x * 4 + threadIdx.x] = v;
    }
}

__global__ void k_energy_m(MGeom g, MCF3 E, MCF3 B, double hv, double *part) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    float f[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int cnt = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nphys; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        phys_ijk(g.n, t, i, j, k);
        int64_t o = (int64_t)i * g.sx + (int64_t)j * g.sy + k;
        int64_t nb[3] = {o + g.sx, o + g.sy, o + 1};
        for (int q = 0; q < 3; q++) {
            const float s = E.p[q][o] + E.p[q][nb[q]];
            f[q] += 0.25f * s * s;
            const float sb = B.p[q][o] + B.p[q][nb[q]];
            f[3 + q] += 0.25f * sb * sb;
        }
        if (++cnt == DIAG_CHUNK) {
            for (int q = 0; q < 6; q++) {
                acc[q] += hv * (double)f[q];
                f[q] = 0.0f;
            }
            cnt = 0;
        }
    }
    for (int q = 0; q < 6; q++) acc[q] += hv * (double)f[q];
    __shared__ double sh[32][6];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 6; q++) {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) v += sh[ww][threadIdx.x];
        part[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

__global__ void k_keys_m(MSpecies st, MState S, int64_t np, int64_t npts, uint32_t *key, uint32_t dead) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    int32_t c = S.cell[p];
    key[p] = c < 0 ? dead : (uint32_t)((int64_t)species_of_m(st, p) * npts + c);
}

// Compaction keys: species index, nspec for removed particles (cell < 0).
__global__ void k_compact_keys_m(MSpecies st, const int32_t *cell, int64_t np, int nspec, uint32_t *key) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    key[p] = cell[p] < 0 ? (uint32_t)nspec : (uint32_t)species_of_m(st, p);
}

// ---- differentiation of the mixed step --------------------------------------
//
// The adjoint of one step of the loop (k_fused_m<REL, false, true> with J
// only, then fold, Yee, executeBC(-1)) for one particle, given the particle
// state before the step (S) and the pack built from the fields before it.
// The forward is recomputed with k_fused_m's own functions (gather_pack,
// push_m, cell_step, axis_bc), so the cell after the step and the boundary
// events are the primal's; cell_after (the state after the step) checks that,
// counting disagreements. L: offset and momentum adjoints, after the step on
// entry, before it on exit. LJ: adjoint of the current at the points (physical
// units; the deposited fixed-point sums are J / q0). LF: the field adjoints,
// which receive the gather's adjoint (atomics; B and B_tm1 each half).
struct MAdjState {
    float *o[3], *u[3];
};
struct MAdjFields {
    float *E[3], *B[3], *T[3];
};
struct MAdjJ {
    const float *J[3];
};
struct MSnapC {
    const int32_t *cell;
    const float *o[3], *u[3];
};

// Adjoint of vb_pieces_list's current for one particle (corrected policy):
// the pieces are placed again with the loop's own operations (crossing
// times by __fdividef, the three-element ordering, fminf, fmaf and
// vb_piece_cell), so each piece lands in the primal's cell; the adjoint of a
// piece's twelve terms is the current adjoint at its cell's points times q0
// (the Jx index of the corrected policy: slot q = 3 at cell + 1); the chain
// goes back through the piece ends and the crossing times to the move's
// start s and end e (old-cell units), added to ls and le. The exit pieces at
// absorbing walls likewise (their wall-plane coordinate is a constant).
__device__ __forceinline__ int vb_point_m(const MGeom &g, int ct, int q) {
    return ct + (q == 3 ? 1 : dep_offset(q, (int)g.sx, (int)g.sy));
}

__device__ void vb_adj_m(const MGeom &g, const BCTab &bc, const MAdjJ &LJ, float q0, const int io[3], const float s[3],
                         const float e[3], float qd, float ls[3], float le[3]) {
    float t[3];
    int ax[3] = {0, 1, 2};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool lo = e[a] < 0.0f, hi = e[a] >= 1.0f;
        t[a] = (lo || hi) ? __fdividef((hi ? 1.0f : 0.0f) - s[a], e[a] - s[a]) : 2.0f;
    }
    // the ordering network of vb_pieces_list, carrying each time's axis
    auto cs = [&](int i, int j) {
        if (t[j] < t[i]) {
            const float tt = t[i];
            t[i] = t[j];
            t[j] = tt;
            const int q = ax[i];
            ax[i] = ax[j];
            ax[j] = q;
        }
    };
    cs(0, 1);
    cs(1, 2);
    cs(0, 1);
    float de[3];
#pragma unroll
    for (int a = 0; a < 3; a++) de[a] = e[a] - s[a];
    float lt[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float ta = k == 0 ? 0.0f : fminf(t[k - 1], 1.0f);
        const float tb = k == 3 ? 1.0f : fminf(t[k], 1.0f);
        if (!(tb > ta)) continue;
        float ua[3], ub[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            ua[a] = fmaf(ta, de[a], s[a]);
            ub[a] = fmaf(tb, de[a], s[a]);
        }
        int c[3];
        const int ct = vb_piece_cell(g, io, ua, ub, c);
        float l[12];
#pragma unroll
        for (int q = 0; q < 12; q++) l[q] = q0 * LJ.J[q >> 2][vb_point_m(g, ct, q)];
        float lua[3] = {0.0f, 0.0f, 0.0f}, lub[3] = {0.0f, 0.0f, 0.0f};
        ad::vb_piece_m_rev(ua, ub, qd, g.ddt, c, l, lua, lub);
        float lta = 0.0f, ltb = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            ls[a] += lua[a] * (1.0f - ta) + lub[a] * (1.0f - tb);
            le[a] += lua[a] * ta + lub[a] * tb;
            lta += lua[a] * de[a];
            ltb += lub[a] * de[a];
        }
        if (k > 0) lt[k - 1] += lta;
        if (k < 3) lt[k] += ltb;
    }
    // a crossing time t = (b - s) / (e - s) of its axis (the others are
    // constants clamped to 1)
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (!(t[k] < 1.0f)) continue;
        const int a = ax[k];
        const float id = __fdividef(1.0f, de[a]);
        ls[a] += lt[k] * (t[k] - 1.0f) * id;
        le[a] += lt[k] * (-t[k] * id);
    }
    const bool absorbs = bc.pbc[0] == PBC_ABSORBING || bc.pbc[1] == PBC_ABSORBING || bc.pbc[2] == PBC_ABSORBING ||
                         bc.pbc[3] == PBC_ABSORBING || bc.pbc[4] == PBC_ABSORBING || bc.pbc[5] == PBC_ABSORBING;
    if (!absorbs) return;
    // the exit pieces: forward to find them, then in reverse
    float A[4][3];
    int dk[3], K = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) A[0][a] = e[a];
    for (int a = 0; a < 3; a++) {
        const bool left = bc.pbc[2 * a] == PBC_ABSORBING && io[a] == 1 && A[K][a] < 0.0f;
        const bool right = bc.pbc[2 * a + 1] == PBC_ABSORBING && io[a] == g.n[a] && A[K][a] >= 1.0f;
        if (!(left || right)) continue;
        for (int b = 0; b < 3; b++) A[K + 1][b] = A[K][b];
        A[K + 1][a] = left ? -1.0f : 2.0f;
        dk[K++] = a;
    }
    float lA[3] = {0.0f, 0.0f, 0.0f};
    for (int k = K - 1; k >= 0; k--) {
        int c[3];
        const int ct = vb_piece_cell(g, io, A[k], A[k + 1], c);
        float l[12];
#pragma unroll
        for (int q = 0; q < 12; q++) l[q] = q0 * LJ.J[q >> 2][vb_point_m(g, ct, q)];
        float la[3] = {0.0f, 0.0f, 0.0f}, lb[3] = {lA[0], lA[1], lA[2]};
        ad::vb_piece_m_rev(A[k], A[k + 1], qd, g.ddt, c, l, la, lb);
        lb[dk[k]] = 0.0f;
        for (int b = 0; b < 3; b++) lA[b] = la[b] + lb[b];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) le[a] += lA[a];
}

// Grid point, relative to the cell, of each of the 18 gather inputs in the
// order of gather_m_weights: Ex F00 F10 F11 F01 over (y, z), Ey over (z, x),
// Ez over (x, y), then the two faces of Bx, By, Bz; 3 bits each (x 4, y 2,
// z 1), input k at bits 3k..3k+2.
constexpr unsigned long long GATHER_CODE =
    (0ull << 0) | (2ull << 3) | (3ull << 6) | (1ull << 9) |       // Ex: o, o+sy, o+sy+1, o+1
    (0ull << 12) | (1ull << 15) | (5ull << 18) | (4ull << 21) |   // Ey: o, o+1, o+sx+1, o+sx
    (0ull << 24) | (4ull << 27) | (6ull << 30) | (2ull << 33) |   // Ez: o, o+sx, o+sx+sy, o+sy
    (0ull << 36) | (4ull << 39) | (0ull << 42) | (2ull << 45) |   // Bx: o, o+sx; By: o, o+sy
    (0ull << 48) | (1ull << 51);                                  // Bz: o, o+1

__device__ __forceinline__ int gather_offset(int k, int sx, int sy) {
    const int c = (int)((GATHER_CODE >> (3 * k)) & 7ull);
    return (c >> 2) * sx + ((c >> 1) & 1) * sy + (c & 1);
}

constexpr int ADJ_BLOCK = 256;
constexpr int ADJ_WARPS = ADJ_BLOCK / 32;
constexpr int GATHER_IN = 18;

// CORR: the corrected policy (true-vertex gather weights, the adjoint of the
// charge-conserving current of the move, also for a particle an absorbing
// wall removed).
template <bool REL, bool CORR>
__global__ void __launch_bounds__(ADJ_BLOCK, CORR ? 3 : 4)
    k_adj_particles_m(MGeom g, Div3 dv, MSpecies st, BCTab bc, const float4 *__restrict__ pack, MSnapC S,
                      const int32_t *cell_after, int64_t np, float q0, MAdjState L, MAdjJ LJ, MAdjFields LF,
                      unsigned long long *mismatch) {
    // per warp: the 18 gather-input adjoints of each lane's particle (a
    // column each), reduced over runs of equal cells before the atomics
    __shared__ float s_g[ADJ_WARPS][GATHER_IN * DEP_STRIDE];
    __shared__ int s_c[ADJ_WARPS][32];
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    float *col = s_g[threadIdx.x >> 5];
    int *keys = s_c[threadIdx.x >> 5];
    int32_t c = -1;
    float lf[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float o_in[3] = {0.0f, 0.0f, 0.0f};
    if (p < np) c = S.cell[p];
    bool zero = false;
    if (!CORR && c >= 0 && cell_after) {
        // every adjoint this particle's step reads is 0 (its offsets and
        // momenta after the step, the current adjoint where it deposited):
        // then so are all it writes, and the recorded cell after the step
        // locates the deposit without recomputing it
        const int32_t ca = cell_after[p];
        zero = ca >= 0;
        if (zero) {
#pragma unroll
            for (int a = 0; a < 3; a++) zero = zero && L.o[a][p] == 0.0f && L.u[a][p] == 0.0f;
        }
        if (zero && st.deposit[species_of_m(st, p)]) {
#pragma unroll
            for (int q = 0; q < 12; q++)
                zero = zero && LJ.J[q >> 2][ca + dep_offset(q, (int)g.sx, (int)g.sy)] == 0.0f;
        }
    }
    if (c >= 0 && !zero) {
        const int s = species_of_m(st, p);
        o_in[0] = S.o[0][p];
        o_in[1] = S.o[1][p];
        o_in[2] = S.o[2][p];
        const float u_in[3] = {S.u[0][p], S.u[1][p], S.u[2][p]};
        int ic[3];
        split_cell(g, dv, c, ic[0], ic[1], ic[2]);
        const float4 *pk = pack + (int64_t)c * PACK_F4;
        float f[6];
        gather_pack(pk, o_in[0], o_in[1], o_in[2], f);
        float u[3] = {u_in[0], u_in[1], u_in[2]}, v[3];
        push_m<REL, false>(f, st.qp[s], nullptr, p, u[0], u[1], u[2], v[0], v[1], v[2]);
        float o[3], nn[3];
        int ii[3] = {ic[0], ic[1], ic[2]};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            nn[a] = o_in[a] + v[a] * g.dtid[a];  // the move's end in the old cell's units
            cell_step(nn[a], ii[a], o[a]);
        }
        // bit a: axis a reflected (u, v -> -u, -v); bit 3 + a: its offset mapped
        // to 1 - o (axis_bc keeps an offset of exactly 0)
        int mask = 0, flip = 0;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (mask & 64) break;
            const float o_pre = o[a];
            const int m = axis_bc(bc, a, g.n[a], ii[a], o[a], u[a], v[a]);
            // static indices into the parameter (a dynamic one copies it to local memory)
            const int kind = ((m >> (2 * a + 1)) & 1) ? bc.pbc[2 * a + 1] : bc.pbc[2 * a];
            if ((m & 63) && !(m & 64) && kind == PBC_REFLECTING) {
                flip |= 1 << a;
                if (o_pre != 0.0f) flip |= 8 << a;
            }
            mask |= m;
        }
        float lo[3] = {0.0f, 0.0f, 0.0f}, lu[3] = {0.0f, 0.0f, 0.0f}, lv[3] = {0.0f, 0.0f, 0.0f};
        float ls[3] = {0.0f, 0.0f, 0.0f};
        const bool removed = (mask & 64) != 0;
        if (!removed) {  // a particle removed in this step leaves nothing after it
            const int32_t onew = ii[0] * (int)g.sx + ii[1] * (int)g.sy + ii[2];
            if (cell_after && cell_after[p] != onew) atomicAdd(mismatch, 1ull);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                lo[a] = L.o[a][p];
                lu[a] = L.u[a][p];
            }
            if (!CORR && st.deposit[s]) {
                float l12[12];
#pragma unroll
                for (int q = 0; q < 12; q++)
                    l12[q] = q0 * LJ.J[q >> 2][onew + dep_offset(q, (int)g.sx, (int)g.sy)];
                ad::jterms_m_rev(st.qdep[s], o, v, l12, lo, lv);
            }
            // boundaries: a reflection maps u -> -u, v -> -v and o -> 1 - o
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (!(flip & (1 << a))) continue;
                lu[a] = -lu[a];
                lv[a] = -lv[a];
                if (flip & (8 << a)) lo[a] = -lo[a];
            }
        }
        if (CORR && st.deposit[s]) {
            // the current of the move (start o_in, end nn, before the boundaries)
            float le[3] = {0.0f, 0.0f, 0.0f};
            vb_adj_m(g, bc, LJ, q0, ic, o_in, nn, st.qdep[s], ls, le);
#pragma unroll
            for (int a = 0; a < 3; a++) lo[a] += le[a];
        }
        if (!removed || CORR) {
            // offset update o' = o + v dt / d (cell held)
#pragma unroll
            for (int a = 0; a < 3; a++) lv[a] += lo[a] * g.dtid[a];
            if (REL) {
                ad::vay_u_rev(st.qp[s], f, u_in, lu, lv, lf);
            } else {
                float lx[3] = {0.0f, 0.0f, 0.0f}, lvb[3] = {lu[0] + lv[0], lu[1] + lv[1], lu[2] + lv[2]};
                ad::boris_rev(st.qp[s], f, 0.0f, u_in, lx, lvb, lf);
#pragma unroll
                for (int a = 0; a < 3; a++) lu[a] = lvb[a];
            }
#pragma unroll
            for (int a = 0; a < 3; a++) lo[a] += ls[a];  // the move's start is the offset before the step
            // gather: the offsets through the pack polynomial
            float pkf[18];
            {
                const float4 ex = pk[0], ey = pk[1], ez = pk[2], bxy = pk[3], bz = pk[4];
                pkf[0] = ex.x; pkf[1] = ex.y; pkf[2] = ex.z; pkf[3] = ex.w;
                pkf[4] = ey.x; pkf[5] = ey.y; pkf[6] = ey.z; pkf[7] = ey.w;
                pkf[8] = ez.x; pkf[9] = ez.y; pkf[10] = ez.z; pkf[11] = ez.w;
                pkf[12] = bxy.x; pkf[13] = bxy.y; pkf[14] = bxy.z; pkf[15] = bxy.w;
                pkf[16] = bz.x; pkf[17] = bz.y;
            }
            ad::gather_m_rev_offsets(pkf, o_in, lf, lo);
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
            L.o[a][p] = lo[a];
            L.u[a][p] = lu[a];
        }
    }
    // the fields through the gather weights, summed over runs of equal cells
    {
        float we[12], wb[6];
        ad::gather_m_weights(o_in, we, wb, CORR);
        float *w = col + lane;
#pragma unroll
        for (int k = 0; k < 12; k++) w[k * DEP_STRIDE] = we[k] * lf[k >> 2];
#pragma unroll
        for (int k = 0; k < 6; k++) w[(12 + k) * DEP_STRIDE] = wb[k] * lf[3 + (k >> 1)];
    }
    const bool active = c >= 0;
    if (__ballot_sync(0xffffffffu, active) == 0u) return;
    const int key = active ? c : -1 - lane;
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != key);
    const unsigned ends = (heads >> 1) | 0x80000000u;  // bit i: particle i ends its run
    keys[lane] = active ? c : -1;
    __syncwarp();
    if (lane < GATHER_IN) {
        const int q = lane;
        const int off = gather_offset(q, (int)g.sx, (int)g.sy);
        // pointer choice by static indices (a dynamic one copies LF to local memory)
        const int cq = q < 12 ? q >> 2 : (q - 12) >> 1;
        float *e = cq == 0 ? LF.E[0] : (cq == 1 ? LF.E[1] : LF.E[2]);
        float *b = cq == 0 ? LF.B[0] : (cq == 1 ? LF.B[1] : LF.B[2]);
        float *t = cq == 0 ? LF.T[0] : (cq == 1 ? LF.T[1] : LF.T[2]);
        float *d0 = q < 12 ? e : b;
        float *d1 = q < 12 ? nullptr : t;
        const float *row = col + q * DEP_STRIDE;
        float acc = 0.0f;
        for (int i = 0; i < 32; i++) {
            acc += row[i];
            if ((ends >> i) & 1u) {
                const int kc = keys[i];
                if (kc >= 0 && acc != 0.0f) {
                    atomicAdd(d0 + (int64_t)kc + off, acc);
                    if (d1) atomicAdd(d1 + (int64_t)kc + off, acc);
                }
                acc = 0.0f;
            }
        }
    }
}

// Selection of the kinetic objective: particles of `species` (-1: all) whose
// x = xyz0 + ((i - 1) + o) dx lies in [xlo, xhi).
struct MKinSel {
    int species;
    double x0, dx, xlo, xhi;
    double m[EMOO_NSPEC];
};

__device__ __forceinline__ bool kin_selected_m(const MGeom &g, const Div3 &dv, const MSpecies &st, const MKinSel &ks,
                                               MSnapC S, int64_t p, int &s) {
    const int32_t c = S.cell[p];
    if (c < 0) return false;
    s = species_of_m(st, p);
    if (ks.species >= 0 && s != ks.species) return false;
    int ix, iy, iz;
    split_cell(g, dv, c, ix, iy, iz);
    const double x = ks.x0 + ((double)(ix - 1) + (double)S.o[0][p]) * ks.dx;
    return x >= ks.xlo && x < ks.xhi;
}

// sum m (gamma - 1) (REL, gamma = sqrt(1 + u^2)) or 0.5 m u^2 over the
// selected particles, in FP64; or, with L, the seed d objective / d u.
template <bool REL>
__global__ void k_kinetic_m(MGeom g, Div3 dv, MSpecies st, MKinSel ks, MSnapC S, int64_t np, double *out,
                            MAdjState L) {
    double a = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        int s;
        if (!kin_selected_m(g, dv, st, ks, S, p, s)) continue;
        const double ux = S.u[0][p], uy = S.u[1][p], uz = S.u[2][p];
        const double u2 = ux * ux + uy * uy + uz * uz, m = ks.m[s];
        if (out) {
            a += REL ? m * (sqrt(1.0 + u2) - 1.0) : 0.5 * m * u2;
        } else {
            const double k = REL ? m / sqrt(1.0 + u2) : m;
            L.u[0][p] += (float)(k * ux);
            L.u[1][p] += (float)(k * uy);
            L.u[2][p] += (float)(k * uz);
        }
    }
    if (!out) return;
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, a);
}

// Before the first push the momentum slots hold the loaded velocity and g0
// the loaded gamma; this stores u = gamma v, the state every later push
// starts from.
__global__ void k_momentum_from_velocity(MState S, const float *g0, int64_t np) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float g = g0[p];
    S.ux[p] *= g;
    S.uy[p] *= g;
    S.uz[p] *= g;
}

// ---- host helpers ----------------------------------------------------------

MGeom mgeom(emoo_handle *h, double dt) {
    MGeom m;
    for (int d = 0; d < 3; d++) {
        m.n[d] = h->g.n[d];
        m.dtid[d] = (float)(dt / h->g.d[d]);
        m.idf[d] = (float)(1.0 / h->g.d[d]);
        m.ddt[d] = dt > 0.0 ? (float)(h->g.d[d] / dt) : 0.0f;
    }
    m.sx = h->g.sx;
    m.sy = h->g.sy;
    m.npts = h->g.npts;
    m.fourpi_dt = (float)(4.0 * PI_D * dt);
    for (int d = 0; d < 3; d++) m.wrap[d] = h->bc.pbc[2 * d] == PBC_PERIODIC ? 1 : 0;
    return m;
}

Div3 div3(emoo_handle *h) {
    Div3 d;
    d.sx = make_fastdiv((uint32_t)h->g.sx);
    d.sy = make_fastdiv((uint32_t)h->g.sy);
    return d;
}

MSpecies mspecies(emoo_handle *h, double dtp) {
    MSpecies st;
    SpeciesTab t;
    species_tab(h, dtp, t);
    st.nspec = t.nspec;
    for (int s = 0; s <= EMOO_NSPEC; s++) st.off[s] = t.off[s];
    for (int s = 0; s < EMOO_NSPEC; s++) {
        st.qp[s] = (float)t.qp[s];
        st.qdep[s] = (float)((t.uq[s] / h->g.vol) / h->mf->q0);
        st.m[s] = (float)t.m[s];
        st.deposit[s] = t.deposit[s];
    }
    return st;
}

MState mstate(emoo_handle *h) { return MState{h->cell, h->ox, h->oy, h->oz, h->ux, h->uy, h->uz}; }

float *mb_role(emoo_handle *h, int c) { return h->bswap ? h->mf->Bslot[3 + c] : h->mf->Bslot[c]; }
float *mt_role(emoo_handle *h, int c) { return h->bswap ? h->mf->Bslot[c] : h->mf->Bslot[3 + c]; }

int nblk(int64_t n, int cap = 152 * 16) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap)); }

}  // namespace

// ---- public (namespace emoo) ----------------------------------------------

int mixed_alloc(emoo_handle *h) {
    // cells are int32 linear indices
    if (h->g.npts >= (int64_t)INT32_MAX) return EMOO_ERR_UNSUPPORTED;
    if (!dep_tables_agree()) return EMOO_ERR_STATE;
    h->mf = new FieldsF32();
    FieldsF32 *m = h->mf;
    size_t n = (size_t)h->g.npts;
    EMOO_CUDA(cudaMalloc(&m->pack, n * PACK_F4 * sizeof(float4)));
    EMOO_CUDA(cudaMalloc(&m->wj, n * DEP_JSLOTS * sizeof(unsigned long long)));
    EMOO_CUDA(cudaMalloc(&m->wr, n * DEP_RSLOTS * sizeof(unsigned long long)));
    for (int c = 0; c < 3; c++) EMOO_CUDA(cudaMalloc(&m->E[c], n * sizeof(float)));
    for (int c = 0; c < 6; c++) EMOO_CUDA(cudaMalloc(&m->Bslot[c], n * sizeof(float)));
    for (int c = 0; c < 4; c++) EMOO_CUDA(cudaMalloc(&m->J[c], n * sizeof(long long)));
    for (int c = 0; c < 3; c++) EMOO_CUDA(cudaMemsetAsync(m->E[c], 0, n * sizeof(float), h->stream));
    for (int c = 0; c < 6; c++) EMOO_CUDA(cudaMemsetAsync(m->Bslot[c], 0, n * sizeof(float), h->stream));
    for (int c = 0; c < 4; c++) EMOO_CUDA(cudaMemsetAsync(m->J[c], 0, n * sizeof(long long), h->stream));
    double qmax = 0.0;
    for (int s = 0; s < h->info.nspecies; s++)
        qmax = std::max(qmax, std::fabs(UNIT_RHOJ * h->info.charge_ratio[s] / h->g.vol));
    if (qmax == 0.0) qmax = 1.0;
    m->q0 = std::ldexp(qmax, -32);
    return EMOO_OK;
}

void mixed_free(emoo_handle *h) {
    FieldsF32 *m = h->mf;
    if (!m) return;
    for (int c = 0; c < 3; c++)
        if (m->E[c]) cudaFree(m->E[c]);
    for (int c = 0; c < 6; c++)
        if (m->Bslot[c]) cudaFree(m->Bslot[c]);
    for (int c = 0; c < 4; c++)
        if (m->J[c]) cudaFree(m->J[c]);
    if (m->pack) cudaFree(m->pack);
    if (m->wj) cudaFree(m->wj);
    if (m->wr) cudaFree(m->wr);
    if (h->g0) cudaFree(h->g0);
    h->g0 = nullptr;
    delete m;
    h->mf = nullptr;
}

// Whether kernels on the handle's device can read and write host array p
// in place: pinned (registered) memory mapped at the same address, device
// or managed memory, or any host memory on a device that uses the host's
// page tables (a coherent CPU-GPU link). Then the conversion kernels move
// the caller's arrays themselves, at the link's bandwidth, without staging.
static bool device_accessible(const emoo_handle *h, const void *p);
bool mixed_device_accessible(const emoo_handle *h, const void *p) { return device_accessible(h, p); }

static bool device_accessible(const emoo_handle *h, const void *p) {
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return a.device == h->dev;
    if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
    int pt = 0;
    if (cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return pt != 0;
}

// n > 0: host FP64 arrays (read in place where the device can, else copied
// through the payload scratch in chunks); n < 0: |n| particles already
// staged on the device at the given pointers.
int mixed_from_f64(emoo_handle *h, int64_t at, int64_t n, const double *x, const double *y, const double *z,
                   const double *vx, const double *vy, const double *vz, const double *gam) {
    bool dev = n < 0;
    if (dev) n = -n;
    if (!dev) {
        const void *src[7] = {x, y, z, vx, vy, vz, gam};
        dev = true;
        for (const void *q : src) dev = dev && device_accessible(h, q);
    }
    int rel = h->info.relativity != 0;
    if (rel && !h->g0) {
        EMOO_CUDA(cudaMalloc(&h->g0, sizeof(float) * (size_t)h->cap));
        h->first_push = 1;  // no push yet: load in velocity mode
    }
    int vmode = rel && h->first_push;
    if (dev) {
        h->launches++;
        k_from_f64<<<nblk(n), 256, 0, h->stream>>>(h->g, mstate(h), at, n, x, y, z, vx, vy, vz, gam, rel, vmode,
                                                   h->g0, h->ctr);
        EMOO_CUDA(cudaGetLastError());
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
        return EMOO_OK;
    }
    int64_t chunk = (int64_t)(h->pay_bytes / (7 * sizeof(double)));
    if (chunk < 1) return EMOO_ERR_OOM;
    double *s = (double *)h->pay;
    for (int64_t b = 0; b < n; b += chunk) {
        int64_t m = std::min(chunk, n - b);
        size_t bytes = sizeof(double) * (size_t)m;
        const double *src[7] = {x, y, z, vx, vy, vz, gam};
        for (int q = 0; q < 7; q++) {
            if (src[q]) EMOO_CUDA(cudaMemcpyAsync(s + q * m, src[q] + b, bytes, cudaMemcpyHostToDevice, h->stream));
        }
        h->launches++;
        k_from_f64<<<nblk(m), 256, 0, h->stream>>>(h->g, mstate(h), at + b, m, s, s + m, s + 2 * m, s + 3 * m,
                                                   s + 4 * m, s + 5 * m, gam ? s + 6 * m : nullptr, rel, vmode,
                                                   h->g0, h->ctr);
        EMOO_CUDA(cudaGetLastError());
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
    }
    return EMOO_OK;
}

int mixed_to_f64(emoo_handle *h, int64_t at, int64_t n, double *x, double *y, double *z, double *vx, double *vy,
                 double *vz, double *gam) {
    int rel = h->info.relativity != 0;
    const float *g0 = (h->first_push && h->g0) ? h->g0 : nullptr;
    bool direct = true;
    for (const void *q : {(const void *)x, (const void *)y, (const void *)z, (const void *)vx, (const void *)vy,
                          (const void *)vz, (const void *)gam})
        direct = direct && device_accessible(h, q);
    if (direct) {  // written in place (see device_accessible)
        h->launches++;
        k_to_f64<<<nblk(n), 256, 0, h->stream>>>(h->g, mstate(h), at, n, x, y, z, vx, vy, vz, gam, rel, g0);
        EMOO_CUDA(cudaGetLastError());
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
        return EMOO_OK;
    }
    int64_t chunk = (int64_t)(h->pay_bytes / (7 * sizeof(double)));
    double *s = (double *)h->pay;
    for (int64_t b = 0; b < n; b += chunk) {
        int64_t m = std::min(chunk, n - b);
        h->launches++;
        k_to_f64<<<nblk(m), 256, 0, h->stream>>>(h->g, mstate(h), at + b, m, s, s + m, s + 2 * m, s + 3 * m,
                                                 s + 4 * m, s + 5 * m, s + 6 * m, rel, g0);
        EMOO_CUDA(cudaGetLastError());
        double *dst[7] = {x, y, z, vx, vy, vz, gam};
        size_t bytes = sizeof(double) * (size_t)m;
        for (int q = 0; q < 7; q++)
            if (dst[q]) EMOO_CUDA(cudaMemcpyAsync(dst[q] + b, s + q * m, bytes, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
    }
    return EMOO_OK;
}

static int mixed_ghost_full(emoo_handle *h, bool e_only);

int mixed_ghost_fill(emoo_handle *h) {
    if (h->policy == EMOO_POLICY_CORRECTED) return mixed_ghost_full(h, false);
    // E/B ghost fill through the fixed storage slots, with LightBC planes for
    // external sides, in the reference's dimension order
    MGeom mg = mgeom(h, h->dtp);
    MList6 fl;
    fl.n = 6;
    for (int c = 0; c < 3; c++) {
        fl.p[c] = h->mf->E[c];
        fl.p[3 + c] = h->mf->Bslot[c];
    }
    const Geom &g = h->g;
    int ta = std::max(g.n[1], g.n[0]);
    int tb = std::max(g.n[2], g.n[1]);
    dim3 blk(32, 8);
    int mask = 0;
    auto flush = [&]() -> int {
        if (!mask) return EMOO_OK;
        dim3 grd((tb + 31) / 32, (ta + 7) / 8, 36);
        h->launches++;
        k_ghost_m<<<grd, blk, 0, h->stream>>>(mg, fl, mask);
        mask = 0;
        EMOO_CUDA(cudaGetLastError());
        return EMOO_OK;
    };
    for (int d = 0; d < 3; d++) {
        if (h->bc.fbc[2 * d] == FBC_PERIODIC) {
            mask |= 1 << d;
            continue;
        }
        EMOO_TRY(flush());
        for (int r = 0; r < 2; r++) {
            int s = 2 * d + r;
            if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
            PlaneSet ps[6];
            int n = light_planes_public(h, s, ps);
            EMOO_TRY(mixed_plane_sets(h, ps, n));
        }
    }
    return flush();
}

// PlaneSet.f carries a field ID (E or B role) for the mixed form.
int mixed_plane_sets(emoo_handle *h, const PlaneSet *ps, int n) {
    MGeom mg = mgeom(h, h->dtp);
    MPlaneList pl;
    pl.n = n;
    for (int i = 0; i < n; i++) {
        int id = (int)(intptr_t)ps[i].f;
        float *f = id < EMOO_BX ? h->mf->E[id] : mb_role(h, id - EMOO_BX);
        pl.s[i] = MPlane{f, ps[i].dim, ps[i].idx, (float)ps[i].v, (float)ps[i].vs, ps[i].t1f, ps[i].t2f};
    }
    const Geom &g = h->g;
    int m = std::max(std::max(g.tot[0], g.tot[1]), g.tot[2]);
    dim3 blk(32, 8);
    dim3 grd((m + 31) / 32, (m + 7) / 8, n);
    h->launches++;
    k_plane_m<<<grd, blk, 0, h->stream>>>(mg, pl, g.tot[0], g.tot[1], g.tot[2]);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// The FP64 form's k_mirror_fold on the fixed-point J (integer adds, exact):
// the current a reflected particle deposited beyond its wall goes to the
// mirrored points inside, normal component negated; ghost values cleared.
__global__ void k_mirror_fold_m(MGeom g, MFix4 fl, int d, int right, int t1, int t2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= t2 || r >= t1) return;
    const int a = blockIdx.z;
    long long *F = fl.p[a];
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int n = g.n[d];
    const bool normal = a == d;
    const int src = normal ? (right ? n + 1 : 0) : (right ? n + 2 : 0);
    const int dst = normal ? (right ? n : 1) : (right ? n : 2);
    int c[3];
    c[o1] = r;
    c[o2] = q;
    c[d] = src;
    const int64_t ks = (int64_t)c[0] * g.sx + (int64_t)c[1] * g.sy + c[2];
    c[d] = dst;
    const int64_t kd = (int64_t)c[0] * g.sx + (int64_t)c[1] * g.sy + c[2];
    if (normal) F[kd] -= F[ks];
    else F[kd] += F[ks];
    F[ks] = 0;
}

// The corrected policy's full-range fold (fixed point) or ghost fill (FP32)
// of n arrays, dimension by dimension: periodic dimensions as images over the
// whole range; walled ones fold J (fix with Jx, Jy, Jz first) by mirror at
// reflecting sides and copy nothing (their field sides are LightBC planes).
static int mixed_periodic_full(emoo_handle *h, const MFix4 *fix, const MF9 *flt, int n) {
    MGeom mg = mgeom(h, h->dtp);
    const Geom &g = h->g;
    dim3 blk(32, 8);
    for (int d = 0; d < 3; d++) {
        const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
        if (h->bc.fbc[2 * d] != FBC_PERIODIC) {
            const bool j3 = fix && n >= 3 && fix->p[0] == h->mf->J[0];
            for (int r = 0; r < 2 && j3; r++) {
                if (h->bc.pbc[2 * d + r] != PBC_REFLECTING) continue;
                dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, 3);
                h->launches++;
                k_mirror_fold_m<<<grd, blk, 0, h->stream>>>(mg, *fix, d, r, g.tot[o1], g.tot[o2]);
            }
            continue;
        }
        dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, n);
        h->launches++;
        if (fix) k_fold_full_m<<<grd, blk, 0, h->stream>>>(mg, *fix, d, g.tot[o1], g.tot[o2]);
        else k_ghost_full_m<<<grd, blk, 0, h->stream>>>(mg, *flt, d, g.tot[o1], g.tot[o2]);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

static int mixed_fold_full(emoo_handle *h, int what) {
    MFix4 fl = {};
    int n = 0;
    if (what & FOLD_J)
        for (int c = 0; c < 3; c++) fl.p[n++] = h->mf->J[c];
    if (what & FOLD_RHO) fl.p[n++] = h->mf->J[3];
    return n ? mixed_periodic_full(h, &fl, nullptr, n) : EMOO_OK;
}

// E (3) or E, B and B_tm1 (9) ghost planes, corrected policy, then the
// LightBC planes of external sides (between the Yee halves too, so that the
// B half reads E at the new time at the boundary planes as at the wrap)
static int mixed_ghost_full(emoo_handle *h, bool e_only) {
    MF9 fl = {};
    for (int c = 0; c < 3; c++) fl.p[c] = h->mf->E[c];
    for (int c = 0; c < 6; c++) fl.p[3 + c] = h->mf->Bslot[c];
    EMOO_TRY(mixed_periodic_full(h, nullptr, &fl, e_only ? 3 : 9));
    for (int s = 0; s < 6; s++) {
        if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
        PlaneSet ps[6];
        const int n = light_planes_public(h, s, ps);
        EMOO_TRY(mixed_plane_sets(h, ps, n));
    }
    return EMOO_OK;
}

// what: FOLD_J (the two transverse J components), FOLD_RHO, or both
static int mixed_fold(emoo_handle *h, int what) {
    if (h->policy == EMOO_POLICY_CORRECTED) return mixed_fold_full(h, what);
    MGeom mg = mgeom(h, h->dtp);
    const Geom &g = h->g;
    for (int d = 0; d < 3; d++) {
        if (h->bc.fbc[2 * d] != FBC_PERIODIC) continue;
        int f0 = (d == 0) ? 1 : 0;  // Jy for x, Jx otherwise
        int f1 = (d == 2) ? 1 : 2;  // Jy for z, Jz otherwise
        int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
        long long *a = h->mf->J[f0], *b = h->mf->J[f1], *r = h->mf->J[3];
        int nz = what == FOLD_J ? 2 : what == FOLD_RHO ? 1 : 3;
        if (what == FOLD_RHO) a = r;
        dim3 blk(32, 8);
        dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, nz);
        h->launches++;
        k_fold_m<<<grd, blk, 0, h->stream>>>(mg, d, a, b, r);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Deposit modes: DEP_J (J only), DEP_J_RHO, DEP_RHO (rho only: J untouched).
constexpr int DEP_J = 0, DEP_J_RHO = 1, DEP_RHO = 2;

// Zeroes the per-cell sums the deposit mode forms its output from; the
// deposit then rewrites Jx, Jy, Jz and / or rho at every point from them.
static int mixed_deposit_zero(emoo_handle *h, int mode) {
    const size_t n = (size_t)h->g.npts * sizeof(unsigned long long);
    if (mode != DEP_RHO) EMOO_CUDA(cudaMemsetAsync(h->mf->wj, 0, n * DEP_JSLOTS, h->stream));
    if (mode != DEP_J) EMOO_CUDA(cudaMemsetAsync(h->mf->wr, 0, n * DEP_RSLOTS, h->stream));
    return EMOO_OK;
}

static int mixed_cells_to_points(emoo_handle *h, int mode) {
    FieldsF32 *m = h->mf;
    const int what = mode == DEP_J ? 1 : mode == DEP_RHO ? 2 : 3;
    h->launches++;
    // four blocks per SM: the neighbouring records a point gathers stay in L2
    // between the points in flight (0.055 ms a step less than eight at 256^3)
    k_cells_to_points<<<nblk(h->g.npts, 152 * 4), 256, 0, h->stream>>>(
        h->g.npts, (int)h->g.sx, (int)h->g.sy, m->wj, m->wr, (unsigned long long *)m->J[0],
        (unsigned long long *)m->J[1], (unsigned long long *)m->J[2], (unsigned long long *)m->J[3], what,
        h->policy == EMOO_POLICY_CORRECTED ? 1 : 0);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// rho += background (fixed point) at the physical points with x index >= i0:
// immobile neutralising ions, no reference counterpart.
__global__ void k_add_phys_i64(MGeom g, long long *f, long long v, int i0) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + i0;
    if (k > g.n[2] || j > g.n[1]) return;
    f[(int64_t)i * g.sx + (int64_t)j * g.sy + k] += v;
}

// J and rho at the points from the per-cell records, plus the background.
static int mixed_finish_deposit(emoo_handle *h, int mode) {
    EMOO_TRY(mixed_cells_to_points(h, mode));
    if (mode == DEP_J || h->opts.rho_background == 0.0 || h->rho_bg_first > h->g.n[0]) return EMOO_OK;
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 grd((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0] - h->rho_bg_first + 1);
    h->launches++;
    k_add_phys_i64<<<grd, blk, 0, h->stream>>>(mgeom(h, h->dtp), h->mf->J[3],
                                               (long long)llrint(h->opts.rho_background / h->mf->q0),
                                               h->rho_bg_first);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Gather + push + boundaries + deposit (push = false: deposit at the current
// state), then J and rho at the points from the per-cell sums. The per-cell
// sums must have been zeroed (mixed_deposit_zero).
static int mixed_fused(emoo_handle *h, double dtp, int mode, bool push = true, bool host = false,
                       int store_pre = 0) {
    const int with_rho = mode != DEP_J ? 1 : 0;
    if (h->np > (int64_t)UINT32_MAX - FUSED_BLOCK) return EMOO_ERR_UNSUPPORTED;  // k_fused_m's 32-bit index
    if (h->np == 0) return mixed_finish_deposit(h, mode);
    MGeom mg = mgeom(h, dtp);
    MSpecies st = mspecies(h, dtp);
    MGather P;
    for (int c = 0; c < 3; c++) {
        P.E[c] = h->mf->E[c];
        P.B[c] = mb_role(h, c);
        P.T[c] = mt_role(h, c);
    }
    MDeposit D;
    D.wj = h->mf->wj;
    D.wr = h->mf->wr;
    int64_t nb = (h->np + FUSED_BLOCK - 1) / FUSED_BLOCK;
    bool rel = h->info.relativity != 0;
    bool first = rel && h->first_push && h->g0;
    Div3 dv = div3(h);
    const float *g0 = h->g0;
    MState S = mstate(h);
    const float4 *pk = h->mf->pack;
    dim3 grd((unsigned)nb);
    const bool corr = h->policy == EMOO_POLICY_CORRECTED;
    if (!push) {
        h->launches++;
#define EMOO_DEPOSIT_M(R, F, C)                                                                                  \
    k_fused_m<R, F, false, C><<<grd, FUSED_BLOCK, 0, h->stream>>>(mg, dv, st, h->bc, pk, S, h->np, D, with_rho, g0, \
                                                                  h->ctr, nullptr, 0)
        if (corr) {
            if (rel && first) EMOO_DEPOSIT_M(true, true, true);
            else if (rel) EMOO_DEPOSIT_M(true, false, true);
            else EMOO_DEPOSIT_M(false, false, true);
        } else {
            if (rel && first) EMOO_DEPOSIT_M(true, true, false);
            else if (rel) EMOO_DEPOSIT_M(true, false, false);
            else EMOO_DEPOSIT_M(false, false, false);
        }
#undef EMOO_DEPOSIT_M
        EMOO_CUDA(cudaGetLastError());
        return mixed_finish_deposit(h, mode);
    }
    {
        const Geom &g = h->g;
        dim3 blk(32, 8);
        dim3 pg((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]);
        h->launches++;
        if (corr) k_pack_m<true><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
        else k_pack_m<false><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
        EMOO_CUDA(cudaGetLastError());
    }
    h->launches++;
    if (h->prof_on) EMOO_CUDA(cudaEventRecord(h->prof_ev[0], h->stream));
#define EMOO_FUSED_M(R, F, C)                                                                                   \
    k_fused_m<R, F, true, C><<<grd, FUSED_BLOCK, 0, h->stream>>>(mg, dv, st, h->bc, pk, S, h->np, D, with_rho, g0, \
                                                                 h->ctr, nullptr, 0)
#define EMOO_FUSED_HOST(R, C)                                                                                    \
    k_fused_m<R, false, true, C, true><<<grd, FUSED_BLOCK, 0, h->stream>>>(mg, dv, st, h->bc, pk, S, h->np, D, 0, \
                                                                           g0, h->ctr, h->mhost, store_pre)
    if (host) {  // the host-resident step: after the first push, J only
        if (corr) {
            if (rel) EMOO_FUSED_HOST(true, true);
            else EMOO_FUSED_HOST(false, true);
        } else {
            if (rel) EMOO_FUSED_HOST(true, false);
            else EMOO_FUSED_HOST(false, false);
        }
    } else if (corr) {
        if (rel && first) EMOO_FUSED_M(true, true, true);
        else if (rel) EMOO_FUSED_M(true, false, true);
        else EMOO_FUSED_M(false, false, true);
    } else {
        if (rel && first) EMOO_FUSED_M(true, true, false);
        else if (rel) EMOO_FUSED_M(true, false, false);
        else EMOO_FUSED_M(false, false, false);
    }
#undef EMOO_FUSED_M
#undef EMOO_FUSED_HOST
    EMOO_CUDA(cudaGetLastError());
    if (h->prof_on) {
        EMOO_CUDA(cudaEventRecord(h->prof_ev[1], h->stream));
        EMOO_TRY(prof_accumulate(h));
    }
    // g0 stays allocated for later loads; it is read only while first_push is set
    if (first) h->first_push = 0;
    return mixed_finish_deposit(h, mode);
}

static int mixed_yee(emoo_handle *h, double dtp, int es) {
    MGeom mg = mgeom(h, dtp);
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 grd((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]);
    MF3 E = {{h->mf->E[0], h->mf->E[1], h->mf->E[2]}};
    MJ3 J = {{h->mf->J[0], h->mf->J[1], h->mf->J[2]}};
    if (es) {
        h->launches++;
        k_yee_es_m<<<grd, blk, 0, h->stream>>>(mg, E, J, (float)dtp, (float)h->mf->q0);
    } else {
        h->bswap ^= 1;  // the member-pointer swap of evolveFields
        MCF3 T = {{mt_role(h, 0), mt_role(h, 1), mt_role(h, 2)}};
        h->launches++;
        k_yee_e_m<<<grd, blk, 0, h->stream>>>(mg, E, T, J, (float)dtp, (float)h->mf->q0);
        // the B half reads E at plane n+1: refreshed first under the corrected
        // policy (time-centred at the periodic wrap, as yee_f64)
        if (h->policy == EMOO_POLICY_CORRECTED) EMOO_TRY(mixed_ghost_full(h, true));
        MF3 B = {{mb_role(h, 0), mb_role(h, 1), mb_role(h, 2)}};
        MCF3 Ec = {{E.p[0], E.p[1], E.p[2]}};
        h->launches++;
        k_yee_b_m<<<grd, blk, 0, h->stream>>>(mg, B, T, Ec, (float)dtp);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// One step of the loop on the host-resident particles (emoo_attach_particles):
// J only, after the first push, without a sort or a history row this step.
// store_pre: the kernel also writes the state it read (before the push) into
// the device store, which then holds what an upload would have left (for the
// history row of this step).
int mixed_step_host(emoo_handle *h, double dtp, int fold_what, int store_pre) {
    if (!h->mhost || (h->info.relativity != 0 && h->first_push)) return EMOO_ERR_STATE;
    EMOO_TRY(mixed_deposit_zero(h, DEP_J));
    EMOO_TRY(mixed_fused(h, dtp, DEP_J, true, true, store_pre));
    EMOO_TRY(mixed_fold(h, fold_what));
    EMOO_TRY(mixed_yee(h, dtp, h->info.electrostatic == 1));
    EMOO_TRY(mixed_ghost_fill(h));
    return EMOO_OK;
}

int mixed_step(emoo_handle *h, double dtp, int with_rho, int fold_what) {
    const int mode = with_rho ? DEP_J_RHO : DEP_J;
    EMOO_TRY(mixed_deposit_zero(h, mode));
    EMOO_TRY(mixed_fused(h, dtp, mode));
    EMOO_TRY(mixed_fold(h, fold_what));
    EMOO_TRY(mixed_yee(h, dtp, h->info.electrostatic == 1));
    EMOO_TRY(mixed_ghost_fill(h));
    return EMOO_OK;
}

int mixed_sort_keys(emoo_handle *h) {
    MSpecies st = mspecies(h, h->dtp);
    uint32_t dead = (uint32_t)((int64_t)h->nspec * h->g.npts + 1);
    h->launches++;
    k_keys_m<<<(unsigned)((h->np + 255) / 256), 256, 0, h->stream>>>(st, mstate(h), h->np, h->g.npts, h->key[0], dead);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_compact_keys(emoo_handle *h) {
    MSpecies st = mspecies(h, h->dtp);
    h->launches++;
    k_compact_keys_m<<<(unsigned)((h->np + 255) / 256), 256, 0, h->stream>>>(st, h->cell, h->np, h->nspec, h->key[0]);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_key_bits(emoo_handle *h) {
    uint64_t maxkey = (uint64_t)h->nspec * (uint64_t)h->g.npts + 2;
    int b = 1;
    while ((1ull << b) <= maxkey) b++;
    return b;
}

// Field readback: FP32 storage or fixed point converted to FP64 in the slot.
int mixed_get_field(emoo_handle *h, int id, double *out_dev) {
    int64_t n = h->g.npts;
    if (id <= EMOO_EZ) k_f2d<<<nblk(n), 256, 0, h->stream>>>(h->mf->E[id], out_dev, n);
    else if (id <= EMOO_BZ) k_f2d<<<nblk(n), 256, 0, h->stream>>>(h->mf->Bslot[id - EMOO_BX], out_dev, n);
    else if (id <= EMOO_RHO) k_fix2d<<<nblk(n), 256, 0, h->stream>>>(h->mf->J[id - EMOO_JX], out_dev, n, h->mf->q0);
    else if (id <= EMOO_BZ_TM1) k_f2d<<<nblk(n), 256, 0, h->stream>>>(h->mf->Bslot[3 + id - EMOO_BX_TM1], out_dev, n);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_set_field(emoo_handle *h, int id, const double *in_dev) {
    int64_t n = h->g.npts;
    if (id <= EMOO_EZ) k_d2f<<<nblk(n), 256, 0, h->stream>>>(in_dev, h->mf->E[id], n);
    else if (id <= EMOO_BZ) k_d2f<<<nblk(n), 256, 0, h->stream>>>(in_dev, h->mf->Bslot[id - EMOO_BX], n);
    else if (id <= EMOO_RHO) k_d2fix<<<nblk(n), 256, 0, h->stream>>>(in_dev, h->mf->J[id - EMOO_JX], n, 1.0 / h->mf->q0);
    else if (id <= EMOO_BZ_TM1) k_d2f<<<nblk(n), 256, 0, h->stream>>>(in_dev, h->mf->Bslot[3 + id - EMOO_BX_TM1], n);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Mixed-form deposit into the FP64 J / rho slots (for the Poisson start):
// one fused pass at dt = 0 is not the reference's deposit (it pushes), so the
// particles are deposited by a zero-step of the FP32 deposit instead.
int mixed_deposit_to_f64(emoo_handle *h) {
    int64_t n = h->g.npts;
    for (int c = 0; c < 4; c++)
        k_fix2d<<<nblk(n), 256, 0, h->stream>>>(h->mf->J[c], h->slot[EMOO_JX + c], n, h->mf->q0);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// After an FP64 field initialisation on the slots: E, B, B_tm1 to FP32.
int mixed_fields_from_slots(emoo_handle *h) {
    int64_t n = h->g.npts;
    for (int c = 0; c < 3; c++) {
        h->launches++;
        k_d2f<<<nblk(n), 256, 0, h->stream>>>(h->slot[EMOO_EX + c], h->mf->E[c], n);
        h->launches++;
        k_d2f<<<nblk(n), 256, 0, h->stream>>>(h->slot[EMOO_BX + c], h->mf->Bslot[c], n);
        h->launches++;
        k_d2f<<<nblk(n), 256, 0, h->stream>>>(h->slot[EMOO_BX_TM1 + c], h->mf->Bslot[3 + c], n);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_const_fields(emoo_handle *h) {
    int64_t n = h->g.npts;
    for (int c = 0; c < 3; c++) {
        h->launches++;
        k_fillf<<<nblk(n), 256, 0, h->stream>>>(h->mf->E[c], n, (float)h->info.E0[c]);
        h->launches++;
        k_fillf<<<nblk(n), 256, 0, h->stream>>>(h->mf->Bslot[c], n, (float)h->info.B0[c]);
        h->launches++;
        k_fillf<<<nblk(n), 256, 0, h->stream>>>(h->mf->Bslot[3 + c], n, (float)h->info.B0[c]);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_moments(emoo_handle *h, double out4[4]) {
    for (int q = 0; q < 4; q++) out4[q] = 0.0;
    if (h->np == 0) return EMOO_OK;
    int nb = nblk(h->np, 152 * 8);
    if (h->red_cap < (size_t)nb * 4) {
        if (h->red) cudaFree(h->red);
        EMOO_CUDA(cudaMalloc(&h->red, (size_t)nb * 4 * sizeof(double)));
        h->red_cap = (size_t)nb * 4;
    }
    MSpecies st = mspecies(h, h->dtp);
    const float *g0 = (h->first_push && h->g0) ? h->g0 : nullptr;
    h->launches++;
    k_moments_m<<<nb, 256, 0, h->stream>>>(st, mstate(h), h->np, h->info.relativity != 0, g0, h->red);
    EMOO_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)nb * 4);
    EMOO_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 4; q++) out4[q] += part[(size_t)b * 4 + q];
    return EMOO_OK;
}

int mixed_field_energy(emoo_handle *h, double out6[6]) {
    const Geom &g = h->g;
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    int nb = nblk(nphys, 152 * 8);
    if (h->red_cap < (size_t)nb * 6) {
        if (h->red) cudaFree(h->red);
        EMOO_CUDA(cudaMalloc(&h->red, (size_t)nb * 6 * sizeof(double)));
        h->red_cap = (size_t)nb * 6;
    }
    MGeom mg = mgeom(h, h->dtp);
    MCF3 E = {{h->mf->E[0], h->mf->E[1], h->mf->E[2]}};
    MCF3 B = {{h->mf->Bslot[0], h->mf->Bslot[1], h->mf->Bslot[2]}};  // fixed slots, like the history
    k_energy_m<<<nb, 256, 0, h->stream>>>(mg, E, B, 0.5 * g.vol, h->red);
    EMOO_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)nb * 6);
    EMOO_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (int q = 0; q < 6; q++) out6[q] = 0.0;
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 6; q++) out6[q] += part[(size_t)b * 6 + q];
    return EMOO_OK;
}

}  // namespace emoo

namespace emoo {

// Particle_Handler::InterpolateEB (src/particles/particle_handler.cpp:138-173)
// for the mixed form: each live particle's E and B from the interpolation
// pack into the FP64 per-particle cache (q * cap + p), as the fused kernel
// gathers them; a removed particle's entries are NaN.
__global__ void k_interpolate_m(const float4 *__restrict__ pack, MState S, int64_t np, int64_t cap, double *fc) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = S.cell[p];
        float f[6];
        if (c >= 0) {
            gather_pack(pack + (int64_t)c * PACK_F4, S.ox[p], S.oy[p], S.oz[p], f);
            for (int q = 0; q < 6; q++) fc[(size_t)q * cap + p] = (double)f[q];
        } else {
            for (int q = 0; q < 6; q++) fc[(size_t)q * cap + p] = __longlong_as_double(0x7ff8000000000000LL);
        }
    }
}

// Particle_Handler::Push with the cached fields (src/particles/particle_handler.cpp:124-128)
// in the mixed form: the fused kernel's push and cell update (push_m,
// cell_step) without the boundaries, which emoo_apply_particle_bc applies. A
// particle may then sit in a ghost cell (0 or n + 1); one that moved further
// is recorded as a bounds error and dropped, as the fused kernel drops it.
template <bool REL, bool FIRST>
__global__ void k_push_cached_m(MGeom g, Div3 dv, MSpecies st, MState S, int64_t np, int64_t cap,
                                const double *__restrict__ fc, const float *g0, DevCounters *ctr) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int32_t c = S.cell[p];
    if (c < 0) return;
    const int s = species_of_m(st, p);
    float f[6];
    for (int q = 0; q < 6; q++) f[q] = (float)fc[(size_t)q * cap + p];
    float ux = S.ux[p], uy = S.uy[p], uz = S.uz[p], vx, vy, vz;
    push_m<REL, FIRST>(f, st.qp[s], g0, p, ux, uy, uz, vx, vy, vz);
    int ix, iy, iz;
    split_cell(g, dv, c, ix, iy, iz);
    float ox = S.ox[p], oy = S.oy[p], oz = S.oz[p];
    cell_step(ox + vx * g.dtid[0], ix, ox);
    cell_step(oy + vy * g.dtid[1], iy, oy);
    cell_step(oz + vz * g.dtid[2], iz, oz);
    if (ix < 0 || ix > g.n[0] + 1 || iy < 0 || iy > g.n[1] + 1 || iz < 0 || iz > g.n[2] + 1) {
        atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
        S.cell[p] = -1;
        return;
    }
    S.cell[p] = ix * (int)g.sx + iy * (int)g.sy + iz;
    S.ox[p] = ox, S.oy[p] = oy, S.oz[p] = oz;
    S.ux[p] = ux, S.uy[p] = uy, S.uz[p] = uz;
}

// executeParticleBoundaryConditions (src/particles/particle_handler.cpp:287-295)
// in the mixed form: the six sides in the fused kernel's order (axis_bc),
// crossings counted per side, removed particles marked.
__global__ void k_particle_bc_m(MGeom g, Div3 dv, BCTab bc, MState S, int64_t np, DevCounters *ctr) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int mask = 0;
    if (p < np && S.cell[p] >= 0) {
        int ix, iy, iz;
        split_cell(g, dv, S.cell[p], ix, iy, iz);
        float o[3] = {S.ox[p], S.oy[p], S.oz[p]}, u[3] = {S.ux[p], S.uy[p], S.uz[p]}, v = 0.0f;
        mask |= axis_bc(bc, 0, g.n[0], ix, o[0], u[0], v);
        if (!(mask & 64)) mask |= axis_bc(bc, 1, g.n[1], iy, o[1], u[1], v);
        if (!(mask & 64)) mask |= axis_bc(bc, 2, g.n[2], iz, o[2], u[2], v);
        if (mask & 64) {
            S.cell[p] = -1;
        } else {
            S.cell[p] = ix * (int)g.sx + iy * (int)g.sy + iz;
            S.ox[p] = o[0], S.oy[p] = o[1], S.oz[p] = o[2];
            S.ux[p] = u[0], S.uy[p] = u[1], S.uz[p] = u[2];
        }
    }
    if (__any_sync(0xffffffffu, mask & 63)) count_cross(ctr, mask & 63);
}

int mixed_push_cached(emoo_handle *h) {
    if (h->np == 0) return EMOO_OK;
    if (!h->fcache) return EMOO_ERR_STATE;
    const bool rel = h->info.relativity != 0, first = rel && h->first_push && h->g0;
    MGeom mg = mgeom(h, h->dtp);
    const unsigned nb = (unsigned)((h->np + 255) / 256);
    h->launches++;
    if (rel && first)
        k_push_cached_m<true, true><<<nb, 256, 0, h->stream>>>(mg, div3(h), mspecies(h, h->dtp), mstate(h), h->np,
                                                               h->cap, h->fcache, h->g0, h->ctr);
    else if (rel)
        k_push_cached_m<true, false><<<nb, 256, 0, h->stream>>>(mg, div3(h), mspecies(h, h->dtp), mstate(h), h->np,
                                                                h->cap, h->fcache, h->g0, h->ctr);
    else
        k_push_cached_m<false, false><<<nb, 256, 0, h->stream>>>(mg, div3(h), mspecies(h, h->dtp), mstate(h), h->np,
                                                                 h->cap, h->fcache, h->g0, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    if (first) h->first_push = 0;
    return EMOO_OK;
}

int mixed_particle_bc(emoo_handle *h) {
    if (h->np == 0) return EMOO_OK;
    h->launches++;
    k_particle_bc_m<<<(unsigned)((h->np + 255) / 256), 256, 0, h->stream>>>(mgeom(h, h->dtp), div3(h), h->bc,
                                                                            mstate(h), h->np, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int mixed_interpolate(emoo_handle *h) {
    if (!h->fcache) EMOO_CUDA(cudaMalloc(&h->fcache, sizeof(double) * 6 * (size_t)h->cap));
    MGeom mg = mgeom(h, h->dtp);
    MGather P;
    for (int c = 0; c < 3; c++) {
        P.E[c] = h->mf->E[c];
        P.B[c] = mb_role(h, c);
        P.T[c] = mt_role(h, c);
    }
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 pg((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]);
    h->launches += 2;
    if (h->policy == EMOO_POLICY_CORRECTED) k_pack_m<true><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
    else k_pack_m<false><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
    if (h->np > 0)
        k_interpolate_m<<<nblk(h->np), 256, 0, h->stream>>>(h->mf->pack, mstate(h), h->np, h->cap, h->fcache);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Particle_Handler::depositRhoJ for the mixed form: zero, then deposit every
// live non-test particle at its current position (no push).
int mixed_deposit(emoo_handle *h, int with_rho) {
    const int mode = with_rho ? DEP_J_RHO : DEP_J;
    EMOO_TRY(mixed_deposit_zero(h, mode));
    return mixed_fused(h, h->dtp, mode, false);
}

// rho alone at the particles' current positions, folded, plus the
// background; J untouched.
int mixed_materialize_rho(emoo_handle *h) {
    EMOO_TRY(mixed_deposit_zero(h, DEP_RHO));
    EMOO_TRY(mixed_fused(h, h->dtp, DEP_RHO, false));
    return mixed_fold(h, FOLD_RHO);
}

int mixed_fold_public(emoo_handle *h) { return mixed_fold(h, FOLD_ALL); }

int mixed_yee_public(emoo_handle *h, double dtp, int es) { return mixed_yee(h, dtp, es); }

// FP32 E, B, B_tm1 and fixed-point J / rho into the FP64 slots (for the FP64
// diagnostics: Gauss-law residual).
int mixed_fields_to_slots(emoo_handle *h) {
    for (int id = 0; id <= EMOO_BZ_TM1; id++) EMOO_TRY(mixed_get_field(h, id, h->slot[id]));
    return EMOO_OK;
}

// ---- differentiation of the mixed step (driven from adjoint_mixed.cu) ----

// The FP32 field storage: E, and the B slots (BX..BZ, BX_TM1..BZ_TM1 storage).
void mixed_field_arrays(emoo_handle *h, float *E[3], float *Bslot[6]) {
    for (int c = 0; c < 3; c++) E[c] = h->mf->E[c];
    for (int c = 0; c < 6; c++) Bslot[c] = h->mf->Bslot[c];
}

// The fixed-point J and rho at the points (Jx, Jy, Jz, rho) and their quantum.
void mixed_point_arrays(emoo_handle *h, long long *J[4], double *q0) {
    for (int c = 0; c < 4; c++) J[c] = h->mf->J[c];
    *q0 = h->mf->q0;
}

// Before the first relativistic push the momentum slots hold the loaded
// velocity (and g0 the loaded gamma); store u = gamma v so that every step
// of a differentiated run is the same function.
int mixed_ad_momentum_from_velocity(emoo_handle *h) {
    if (!(h->info.relativity && h->first_push && h->g0)) return EMOO_OK;
    if (h->np) {
        h->launches++;
        k_momentum_from_velocity<<<(unsigned)((h->np + 255) / 256), 256, 0, h->stream>>>(mstate(h), h->g0, h->np);
        EMOO_CUDA(cudaGetLastError());
    }
    h->first_push = 0;
    return EMOO_OK;
}

int mixed_ad_particles(emoo_handle *h, const MSnapView &S, const int32_t *cell_after, float *const lo[3],
                       float *const lu[3], const float *const lj[3], float *const lE[3], float *const lB[3],
                       float *const lT[3], unsigned long long *mismatch) {
    if (h->np == 0) return EMOO_OK;
    MGeom mg = mgeom(h, h->dtp);
    {
        MGather P;
        for (int c = 0; c < 3; c++) {
            P.E[c] = S.E[c];
            P.B[c] = S.B[c];
            P.T[c] = S.T[c];
        }
        const Geom &g = h->g;
        dim3 blk(32, 8);
        dim3 pg((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]);
        h->launches++;
        if (h->policy == EMOO_POLICY_CORRECTED) k_pack_m<true><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
        else k_pack_m<false><<<pg, blk, 0, h->stream>>>(mg, P, h->mf->pack);
        EMOO_CUDA(cudaGetLastError());
    }
    MSnapC SC{S.cell, {S.o[0], S.o[1], S.o[2]}, {S.u[0], S.u[1], S.u[2]}};
    MAdjState L{{lo[0], lo[1], lo[2]}, {lu[0], lu[1], lu[2]}};
    MAdjJ LJ{{lj[0], lj[1], lj[2]}};
    MAdjFields LF{{lE[0], lE[1], lE[2]}, {lB[0], lB[1], lB[2]}, {lT[0], lT[1], lT[2]}};
    MSpecies st = mspecies(h, h->dtp);
    Div3 dv = div3(h);
    const float q0 = (float)h->mf->q0;
    const unsigned nb = (unsigned)((h->np + 255) / 256);
    h->launches++;
    const bool corr = h->policy == EMOO_POLICY_CORRECTED;
#define EMOO_ADJ_M(R, C) \
    k_adj_particles_m<R, C><<<nb, 256, 0, h->stream>>>(mg, dv, st, h->bc, h->mf->pack, SC, cell_after, h->np, q0, L, LJ, \
                                                       LF, mismatch)
    if (h->info.relativity) {
        if (corr) EMOO_ADJ_M(true, true);
        else EMOO_ADJ_M(true, false);
    } else {
        if (corr) EMOO_ADJ_M(false, true);
        else EMOO_ADJ_M(false, false);
    }
#undef EMOO_ADJ_M
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// The kinetic objective of the particles in state S (dev_out: += its value)
// or its seed (lu += d objective / d u).
int mixed_ad_kinetic(emoo_handle *h, const MSnapView &S, int species, double xlo, double xhi, double *dev_out,
                     float *const lu[3]) {
    if (h->np == 0) return EMOO_OK;
    MKinSel ks;
    ks.species = species;
    ks.x0 = h->info.xyz0[0];
    ks.dx = h->g.d[0];
    ks.xlo = xlo;
    ks.xhi = xhi;
    for (int s = 0; s < EMOO_NSPEC; s++) ks.m[s] = h->info.mass_ratio[s];
    MSnapC SC{S.cell, {S.o[0], S.o[1], S.o[2]}, {S.u[0], S.u[1], S.u[2]}};
    MAdjState L{{nullptr, nullptr, nullptr}, {lu ? lu[0] : nullptr, lu ? lu[1] : nullptr, lu ? lu[2] : nullptr}};
    MGeom mg = mgeom(h, h->dtp);
    MSpecies st = mspecies(h, h->dtp);
    Div3 dv = div3(h);
    const int nb = nblk(h->np);
    h->launches++;
    if (h->info.relativity)
        k_kinetic_m<true><<<nb, 256, 0, h->stream>>>(mg, dv, st, ks, SC, h->np, lu ? nullptr : dev_out, L);
    else
        k_kinetic_m<false><<<nb, 256, 0, h->stream>>>(mg, dv, st, ks, SC, h->np, lu ? nullptr : dev_out, L);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

}  // namespace emoo
