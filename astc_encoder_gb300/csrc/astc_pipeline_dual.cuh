// astc_pipeline_dual.cuh -- dual-plane candidates of the FP32 encoder's
// quality modes from ASTC_QUALITY_THOROUGH up.  The reference
// shader writes the dual-plane bit of its block mode as a constant 0
// (assemble_blockmode, ASTC_Encode.hlsl:446-473).
//
// Plane 2 carries one channel pc.  For each channel that varies over the
// block, the shader's power iteration runs on the block's covariance with that
// channel's row and column zeroed (the PCA of the block with the channel held
// constant; the axis's component on the channel is then exactly 0, so it takes
// no part in find_min_max's projections).  pc is the channel whose zeroed
// covariance keeps the least off-axis variance: its trace minus the Rayleigh
// quotient v.Cv / v.v (the first channel on ties) -- or, when fewer than
// three channels vary (a normal map's x and y), the first varying channel.
// The other channels are fitted on pc's axis, pc's endpoints are its minimum
// and maximum.  Every weight range whose 32 weights (plane 1, plane 2
// per grid point; 24..96 bits) leave a legal endpoint range after the 2-bit
// plane selector is scored by the exact decode, each channel taking its
// plane's weight.  Plane-1 weights project the grid colours on the decoded
// endpoints without pc, plane-2 weights are (c_pc - E0_pc) / (E1_pc - E0_pc),
// both clamped to [0, 1] and rounded to the range.  The oracle's dual_plane
// follows the same steps.
#pragma once
#include "astc_pipeline_search.cuh"

namespace astc {

// Per-CTA copies of the dual-plane endpoint tables (shared memory).
struct DualSmem {
    uint16_t color[8][256];
    int8_t cq[12];       // weight range -> endpoint range (-1: illegal)
    int8_t slot[12];
};

// The squared error of a dual-plane decode (channel pc on plane-2 weights).
// P[g]: grid point g's unquantised plane-1 weight in the low half, its plane-2
// weight in the high half (each 0..64, so the 6x6 infill sums, at most
// 64 * 16, stay inside their halves and are computed on both at once).
template <int DIM, bool ALPHA, bool SRGB>
__device__ __forceinline__ uint32_t eval_dual(const uint32_t (&tw)[DIM * DIM], uint32_t t2, int pc, const int E0[4],
                                              const int E1[4], const uint32_t (&P)[16]) {
    constexpr int NCH = ALPHA ? 4 : 3;
    int base[NCH], delta[NCH];
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
        const int c0 = SRGB ? ((E0[c] << 8) | 0x80) : E0[c] * 257;
        const int c1 = SRGB ? ((E1[c] << 8) | 0x80) : E1[c] * 257;
        base[c] = 4 * (64 * c0 + 32);
        delta[c] = 4 * (c1 - c0);
    }
    uint32_t dd = 0, dt = 0;
#pragma unroll
    for (int k = 0; k < DIM * DIM; ++k) {
        int w1, w2;
        if constexpr (DIM == 6) {
            const Infill f = infill_6x6(k);
            uint32_t a = P[f.v0] * (uint32_t)f.w00 + 0x00080008u;
            if (f.w01) a += P[f.v0 + 1] * (uint32_t)f.w01;
            if (f.w10) a += P[f.v0 + 4] * (uint32_t)f.w10;
            if (f.w11) a += P[f.v0 + 5] * (uint32_t)f.w11;
            w1 = (int)((a & 0xFFFFu) >> 4);
            w2 = (int)(a >> 20);
        } else {
            w1 = (int)(P[k] & 0xFFFFu);
            w2 = (int)(P[k] >> 16);
        }
        uint32_t v[NCH];
#pragma unroll
        for (int c = 0; c < NCH; ++c) v[c] = (uint32_t)(base[c] + delta[c] * (c == pc ? w2 : w1));
        uint32_t dec = __byte_perm(v[0], v[1], 0x3362u);
        dec = __byte_perm(dec, v[2], 0x3610u);
        if constexpr (ALPHA) dec = __byte_perm(dec, v[3], 0x6210u);
        dd = __dp4a(dec, dec, dd);
        dt = __dp4a(dec, tw[k], dt);
    }
    return dd - 2u * dt + t2;
}

// One dual-plane block: mode with D (bit 10) set, CEM [16:13], endpoints from
// bit 17, the plane selector right below the weights, 32 interleaved weights
// bit-reversed from bit 127.
template <bool ALPHA>
__device__ __forceinline__ uint4 assemble_dual(int wq, int cq, int pc, const uint32_t (&ev)[ALPHA ? 8 : 6],
                                               const uint32_t (&sw)[32], const SearchSmem& sm) {
    const Bits128 ep = ise_encode_endpoints<ALPHA ? 8 : 6>(cq, ev, sm.trits, sm.quints);
    const Bits128 wt = ise_encode_weights<32, kQuant2, kQuant6>(wq, sw, sm.trits, sm.quints);
    const int sel = 128 - ise_bit_count(wq, 32) - 2;       // 32..102: never straddles the words
    const uint64_t head = (uint64_t)blockmode_4x4_grid(wq) | (1ull << 10) | ((uint64_t)(ALPHA ? 12u : 8u) << 13);
    uint64_t lo = head | (ep.lo << 17) | __brevll(wt.hi);
    uint64_t hi = (ep.lo >> 47) | (ep.hi << 17) | __brevll(wt.lo);
    if (sel < 64) lo |= (uint64_t)pc << sel;
    else hi |= (uint64_t)pc << (sel - 64);
    return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

// Dual-plane candidates of one block; returns `best` unless one decodes with
// less error than best_err (which it then lowers).  st: the fit-space texels,
// grid: the 16 grid-point colours, tw/t2: the scoring targets.
template <int DIM, bool ALPHA, bool SRGB, class S, class G>
__device__ __forceinline__ uint4 dual_plane_block(const S& st, const G& grid, const uint32_t (&tw)[DIM * DIM],
                                                  uint32_t t2, uint32_t& best_err, uint4 best, const SearchSmem& sm,
                                                  const DualSmem& ds) {
    constexpr int N = DIM * DIM;
    constexpr int NCH = ALPHA ? 4 : 3;
    const float4 m = block_mean<N>(st);
    const Covariance cv = block_covariance<N>(st, m);
    // each channel's range (one pass); constant channels have nothing to split off
    float lo[4] = {1e31f, 1e31f, 1e31f, 1e31f}, hi[4] = {-1e31f, -1e31f, -1e31f, -1e31f};
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float4 t = st.get(k);
        lo[0] = fminf(lo[0], t.x); hi[0] = fmaxf(hi[0], t.x);
        lo[1] = fminf(lo[1], t.y); hi[1] = fmaxf(hi[1], t.y);
        lo[2] = fminf(lo[2], t.z); hi[2] = fmaxf(hi[2], t.z);
        if constexpr (ALPHA) { lo[3] = fminf(lo[3], t.w); hi[3] = fmaxf(hi[3], t.w); }
    }
    int nvary = 0, first = -1;
#pragma unroll
    for (int c = 0; c < NCH; ++c)
        if (lo[c] != hi[c]) {
            ++nvary;
            if (first < 0) first = c;
        }
    if (nvary == 0) return best;
    // the plane-2 channel: with three or more varying, the one whose zeroed
    // covariance keeps the least off-axis variance (first on ties); with fewer
    // (a normal map's x and y), the first varying channel
    int pc = first;
    float4 pv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float least = 0.0f;
#pragma unroll 1
    for (int c = nvary < 3 ? first : 0; c < (nvary < 3 ? first + 1 : NCH); ++c) {
        const float clo = c == 0 ? lo[0] : c == 1 ? lo[1] : c == 2 ? lo[2] : lo[3];
        const float chi = c == 0 ? hi[0] : c == 1 ? hi[1] : c == 2 ? hi[2] : hi[3];
        if (clo == chi) continue;
        // entry (i, j) is zeroed when i or j is c
        const bool z0 = c == 0, z1 = c == 1, z2 = c == 2, z3 = c == 3;
        const float a00 = z0 ? 0.0f : cv.c00, a01 = (z0 || z1) ? 0.0f : cv.c01;
        const float a02 = (z0 || z2) ? 0.0f : cv.c02, a03 = (z0 || z3) ? 0.0f : cv.c03;
        const float a11 = z1 ? 0.0f : cv.c11, a12 = (z1 || z2) ? 0.0f : cv.c12;
        const float a13 = (z1 || z3) ? 0.0f : cv.c13, a22 = z2 ? 0.0f : cv.c22;
        const float a23 = (z2 || z3) ? 0.0f : cv.c23, a33 = z3 ? 0.0f : cv.c33;
        const float4 v = power_iteration(a00, a01, a02, a03, a11, a12, a13, a22, a23, a33);
        if (nvary < 3) {
            pv = v;
            break;
        }
        // trace minus the Rayleigh quotient v.Cv / v.v
        const float k0 = dot4(a00, a01, a02, a03, v.x, v.y, v.z, v.w);
        const float k1 = dot4(a01, a11, a12, a13, v.x, v.y, v.z, v.w);
        const float k2 = dot4(a02, a12, a22, a23, v.x, v.y, v.z, v.w);
        const float k3 = dot4(a03, a13, a23, a33, v.x, v.y, v.z, v.w);
        const float vv = dot4(v.x, v.y, v.z, v.w, v.x, v.y, v.z, v.w);
        const float lam = vv > 0.0f ? __fdiv_rn(dot4(v.x, v.y, v.z, v.w, k0, k1, k2, k3), vv) : 0.0f;
        const float resid = __fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(a00, a11), a22), a33), lam);
        if (c == first || resid < least) { pc = c; least = resid; pv = v; }
    }
    const float plo = pc == 0 ? lo[0] : pc == 1 ? lo[1] : pc == 2 ? lo[2] : lo[3];
    const float phi = pc == 0 ? hi[0] : pc == 1 ? hi[1] : pc == 2 ? hi[2] : hi[3];
    // the other channels on pc's axis (its pc component is exactly 0), pc on
    // its range
    uint32_t q0[4], q1[4];
    {
        float e0[4], e1[4];
        find_min_max<N, ALPHA>(st, m, pv, e0, e1, q0, q1);
    }
    const uint32_t lq = rint_u32(plo), hq = rint_u32(phi);
    q0[0] = pc == 0 ? lq : q0[0]; q0[1] = pc == 1 ? lq : q0[1]; q0[2] = pc == 2 ? lq : q0[2];
    q0[3] = pc == 3 ? lq : q0[3];
    q1[0] = pc == 0 ? hq : q1[0]; q1[1] = pc == 1 ? hq : q1[1]; q1[2] = pc == 2 ? hq : q1[2];
    q1[3] = pc == 3 ? hq : q1[3];
    // every legal weight range, then one more pass over the best to assemble it
    int found = -1;
    uint4 out = best;
#pragma unroll 1
    for (int it = kQuant2; it <= kQuant32 + 1; ++it) {
        const bool final_pass = it > kQuant32;
        if (final_pass && found < 0) break;
        const int wq = final_pass ? found : it;
        const int cq = ds.cq[wq];
        if (cq < 0) continue;
        int sym0[4], sym1[4], E0[4], E1[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) { sym0[c] = 0; sym1[c] = 0; E0[c] = 255; E1[c] = 255; }
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            if (cq == kQuant256) {
                sym0[c] = E0[c] = (int)q0[c];
                sym1[c] = E1[c] = (int)q1[c];
            } else {
                const uint32_t a = ds.color[ds.slot[wq]][q0[c]], b = ds.color[ds.slot[wq]][q1[c]];
                sym0[c] = (int)(a & 0xFFu); E0[c] = (int)(a >> 8);
                sym1[c] = (int)(b & 0xFFu); E1[c] = (int)(b >> 8);
            }
        }
        if (E1[0] + E1[1] + E1[2] < E0[0] + E0[1] + E0[2]) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                int t = sym0[c]; sym0[c] = sym1[c]; sym1[c] = t;
                t = E0[c]; E0[c] = E1[c]; E1[c] = t;
            }
        }
        float d[4], f[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            f[c] = (float)E0[c];
            d[c] = c == pc ? 0.0f : (float)(E1[c] - E0[c]);
        }
        const float dd = dot4(d[0], d[1], d[2], d[3], d[0], d[1], d[2], d[3]);
        const float r = dd == 0.0f ? 0.0f : __frcp_rn(dd);
        // selects, not E[pc]: a runtime index would put E0/E1 in local memory
        const int e0p = pc == 0 ? E0[0] : pc == 1 ? E0[1] : pc == 2 ? E0[2] : E0[3];
        const int e1p = pc == 0 ? E1[0] : pc == 1 ? E1[1] : pc == 2 ? E1[2] : E1[3];
        const float dp = (float)(e1p - e0p);
        const float rp = dp == 0.0f ? 0.0f : __frcp_rn(dp);
        const float R = sm.wmax[wq];
        // scoring passes: the weights' values; the final pass: their ISE symbols
        const uint8_t* tab = final_pass ? sm.scramble[wq] : sm.wval[wq];
        uint32_t P[16];
#pragma unroll
        for (int g = 0; g < 16; ++g) {
            const float4 sg = grid.get(g);
            const float x0 = __fsub_rn(sg.x, f[0]), x1 = __fsub_rn(sg.y, f[1]);
            const float x2 = __fsub_rn(sg.z, f[2]), x3 = __fsub_rn(sg.w, f[3]);
            const float w1 = fminf(fmaxf(__fmul_rn(dot4(x0, x1, x2, x3, d[0], d[1], d[2], d[3]), r), 0.0f), 1.0f);
            const float xp = pc == 0 ? x0 : pc == 1 ? x1 : pc == 2 ? x2 : x3;
            const float w2 = fminf(fmaxf(__fmul_rn(xp, rp), 0.0f), 1.0f);
            P[g] = (uint32_t)tab[rint_u32(__fmul_rn(w1, R))] | ((uint32_t)tab[rint_u32(__fmul_rn(w2, R))] << 16);
        }
        if (!final_pass) {
            const uint32_t err = eval_dual<DIM, ALPHA, SRGB>(tw, t2, pc, E0, E1, P);
            if (err < best_err) { best_err = err; found = wq; }
            continue;
        }
        uint32_t ev[ALPHA ? 8 : 6];
#pragma unroll
        for (int c = 0; c < NCH; ++c) { ev[2 * c] = (uint32_t)sym0[c]; ev[2 * c + 1] = (uint32_t)sym1[c]; }
        uint32_t sw[32];
#pragma unroll
        for (int g = 0; g < 16; ++g) { sw[2 * g] = P[g] & 0xFFFFu; sw[2 * g + 1] = P[g] >> 16; }
        out = assemble_dual<ALPHA>(wq, cq, pc, ev, sw, sm);
        break;
    }
    return out;
}

}  // namespace astc
