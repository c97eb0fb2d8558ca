// Packed FP32 arithmetic (Blackwell f32x2: add/sub/mul/fma on a pair of floats per instruction)
// and the Fenton-Karma cell arithmetic restated on pairs of cells.
//
// Every packed function performs, lane by lane, exactly the operations of its scalar
// counterpart in fk_math.cuh in the same order and rounding (.rn, no flush-to-zero), so a cell
// computed here is bit-identical to the same cell computed by the scalar kernels.  Signs are
// folded into constants only where IEEE arithmetic makes that exact: -(a * b) == a * (-b) and
// (-a) * b == -(a * b) under round-to-nearest.
//
// Constants come from a __grid_constant__ kernel parameter (PackConsts) so that they are read
// as constant-bank operands instead of occupying a register pair each.
//
// Contraction hazard.  The assembler may fuse a packed multiply into a following packed add
// (one rounding instead of two) even though both carry an explicit .rn, which the scalar
// kernels, built with --fmad=false, never do.  Every sum whose operand is the result of a packed
// multiply is therefore written so that no multiply->add pair exists: as fma(1, a, product)
// (p_add_product: exact, since 1*a is exact, and a product in the addend slot cannot be fused)
// when the other operand is not itself a product, or as two scalar adds when both are.
#pragma once
#include <cuda_runtime.h>

#include "fk_math.cuh"

namespace fk {

__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 p_add(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mk2(float x, float y) { return make_float2(x, y); }
// a + b for two products (scalar adds: nothing to fuse)
__device__ __forceinline__ float2 add_products(float2 a, float2 b) { return mk2(a.x + b.x, a.y + b.y); }

// Pair constants of one launch (host-built; every field holds the same value twice).
struct PackConsts {
    // cardiax/solve.py:232-249 stencil coefficients, signs as used by g_central/g_head/g_tail
    float2 c_1_12, c_m2_3, c_2_3, c_m1_12;     // central rows
    float2 c_head0, c_three, c_m3_2, c_1_3;    // first two rows
    float2 c_tail0, c_3_2, c_mthree, c_tail3;  // last two rows
    float2 rdx, dt, one, two, m2log2e;
    // model (cardiax/params.py), with the signs of fk::reaction folded in
    float2 V_c, V_csi, k, neg_r_tau_d, r_tau_0, neg_r_2tau_si, neg_r_Cm, neg_r_tau_vp,
        neg_r_tau_wp, r_tau_wm;
};

inline PackConsts make_pack_consts(const Model &m, float rdx, float dt) {
    auto d = [](float x) { return float2{x, x}; };
    PackConsts k;
    k.c_1_12 = d(C_1_12);
    k.c_m2_3 = d(-C_2_3);
    k.c_2_3 = d(C_2_3);
    k.c_m1_12 = d(-C_1_12);
    k.c_head0 = d(C_HEAD0);
    k.c_three = d(C_THREE);
    k.c_m3_2 = d(-C_3_2);
    k.c_1_3 = d(C_1_3);
    k.c_tail0 = d(C_TAIL0);
    k.c_3_2 = d(C_3_2);
    k.c_mthree = d(-C_THREE);
    k.c_tail3 = d(C_TAIL3);
    k.rdx = d(rdx);
    k.dt = d(dt);
    k.one = d(1.0f);
    k.two = d(2.0f);
    k.m2log2e = d(-2.8853900817779268f);  // the constant of fk::one_plus_tanh
    k.V_c = d(m.V_c);
    k.V_csi = d(m.V_csi);
    k.k = d(m.k);
    k.neg_r_tau_d = d(-m.r_tau_d);
    k.r_tau_0 = d(m.r_tau_0);
    k.neg_r_2tau_si = d(-m.r_2tau_si);
    k.neg_r_Cm = d(-m.r_Cm);
    k.neg_r_tau_vp = d(-m.r_tau_vp);
    k.neg_r_tau_wp = d(-m.r_tau_wp);
    k.r_tau_wm = d(m.r_tau_wm);
    return k;
}

// a + product, where `product` is the result of a packed multiply (see the contraction hazard).
__device__ __forceinline__ float2 p_add_product(const PackConsts &k, float2 a, float2 product) {
    return p_fma(k.one, a, product);
}

// g_central / g_head / g_tail of fk_math.cuh on a pair of lines.
__device__ __forceinline__ float2 pg_central(const PackConsts &k, float2 m2, float2 m1, float2 p1,
                                             float2 p2) {
    float2 s = p_mul(k.c_1_12, m2);
    s = p_fma(k.c_m2_3, m1, s);
    s = p_fma(k.c_2_3, p1, s);
    return p_fma(k.c_m1_12, p2, s);
}
__device__ __forceinline__ float2 pg_head(const PackConsts &k, float2 a0, float2 a1, float2 a2,
                                          float2 a3) {
    float2 s = p_mul(k.c_head0, a0);
    s = p_fma(k.c_three, a1, s);
    s = p_fma(k.c_m3_2, a2, s);
    return p_fma(k.c_1_3, a3, s);
}
__device__ __forceinline__ float2 pg_tail(const PackConsts &k, float2 a0, float2 a1, float2 a2,
                                          float2 a3) {
    float2 s = p_mul(k.c_tail0, a0);
    s = p_fma(k.c_3_2, a1, s);
    s = p_fma(k.c_mthree, a2, s);
    return p_fma(k.c_tail3, a3, s);
}

// pg_central over the pairs (a0, a1), (a1, a2), (a3, a4), (a4, a5) -- the central stencil of two
// neighbouring cells along a row -- when only (a0, a1) and (a4, a5) sit in register-aligned pairs:
// the two middle taps as scalar fmas, the same operations per lane in the same order, so no
// register moves are needed to form the misaligned pairs.
__device__ __forceinline__ float2 pg_central_row(const PackConsts &k, float a0, float a1, float a2,
                                                 float a3, float a4, float a5) {
    float2 s = p_mul(k.c_1_12, mk2(a0, a1));
    s.x = fmaf(k.c_m2_3.x, a1, s.x);
    s.y = fmaf(k.c_m2_3.x, a2, s.y);
    s.x = fmaf(k.c_2_3.x, a3, s.x);
    s.y = fmaf(k.c_2_3.x, a4, s.y);
    return p_fma(k.c_m1_12, mk2(a4, a5), s);
}

// A quad of 4 consecutive columns held as two pairs (c, c+1) and (c+2, c+3).
struct Quad {
    float2 lo, hi;
};
__device__ __forceinline__ Quad ld_quad(const float *p) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    return Quad{mk2(v.x, v.y), mk2(v.z, v.w)};
}
__device__ __forceinline__ Quad q_central(const PackConsts &k, const Quad &m2, const Quad &m1,
                                          const Quad &p1, const Quad &p2) {
    return Quad{pg_central(k, m2.lo, m1.lo, p1.lo, p2.lo), pg_central(k, m2.hi, m1.hi, p1.hi, p2.hi)};
}
__device__ __forceinline__ Quad q_head(const PackConsts &k, const Quad &a0, const Quad &a1,
                                       const Quad &a2, const Quad &a3) {
    return Quad{pg_head(k, a0.lo, a1.lo, a2.lo, a3.lo), pg_head(k, a0.hi, a1.hi, a2.hi, a3.hi)};
}
__device__ __forceinline__ Quad q_tail(const PackConsts &k, const Quad &a0, const Quad &a1,
                                       const Quad &a2, const Quad &a3) {
    return Quad{pg_tail(k, a0.lo, a1.lo, a2.lo, a3.lo), pg_tail(k, a0.hi, a1.hi, a2.hi, a3.hi)};
}
__device__ __forceinline__ Quad q_scale(const Quad &a, float2 s) {
    return Quad{p_mul(a.lo, s), p_mul(a.hi, s)};
}

__device__ __forceinline__ float ex2_approx(float x) {
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x));
    return e;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// fk::reaction on two cells (cardiax/solve.py:34-42,57-58).
struct PairReaction {
    float2 dv, dw, j_ion;
};
__device__ __forceinline__ PairReaction p_reaction(const PackConsts &k, const Model &m, float2 u,
                                                   float2 v, float2 w) {
    const bool p0 = u.x >= m.V_c, p1 = u.y >= m.V_c;
    const bool q0 = u.x >= m.V_v, q1 = u.y >= m.V_v;
    // j_fi = -v p (u - V_c)(1 - u) / tau_d
    const float2 jfi_on = p_mul(p_mul(p_mul(v, p_sub(u, k.V_c)), p_sub(k.one, u)), k.neg_r_tau_d);
    // j_so = u (1 - p) / tau_0 + p / tau_r
    const float2 jso_off = p_mul(u, k.r_tau_0);
    const float2 jfs = p_add(mk2(p0 ? jfi_on.x : 0.0f, p1 ? jfi_on.y : 0.0f),
                             mk2(p0 ? m.inv_tau_r : jso_off.x, p1 ? m.inv_tau_r : jso_off.y));
    // j_si = -w (1 + tanh(k (u - V_csi))) / (2 tau_si), 1 + tanh(x) = 2 / (1 + 2^(x * -2/ln 2))
    const float2 xe = p_mul(p_mul(k.k, p_sub(u, k.V_csi)), k.m2log2e);
    const float2 ope = p_add(k.one, mk2(ex2_approx(xe.x), ex2_approx(xe.y)));
    const float2 opt = p_mul(k.two, mk2(rcp_approx(ope.x), rcp_approx(ope.y)));
    const float2 jsi = p_mul(p_mul(w, opt), k.neg_r_2tau_si);
    PairReaction r;
    r.j_ion = p_mul(p_add_product(k, jfs, jsi), k.neg_r_Cm);
    const float2 dv_on = p_mul(v, k.neg_r_tau_vp);
    const float2 dv_off = p_mul(p_sub(k.one, v), mk2(q0 ? m.r_tau_v2m : m.r_tau_v1m,
                                                     q1 ? m.r_tau_v2m : m.r_tau_v1m));
    const float2 dw_on = p_mul(w, k.neg_r_tau_wp);
    const float2 dw_off = p_mul(p_sub(k.one, w), k.r_tau_wm);
    r.dv = mk2(p0 ? dv_on.x : dv_off.x, p1 ? dv_on.y : dv_off.y);
    r.dw = mk2(p0 ? dw_on.x : dw_off.x, p1 ? dw_on.y : dw_off.y);
    return r;
}

}  // namespace fk
