// Per-cell Fenton-Karma arithmetic shared by every kernel of the library.
//
// All kernels (plain step, temporally blocked step, batched persistent step, adjoint recompute)
// call these functions, and the library is compiled with --fmad=false, so every fused
// multiply-add below is explicit and every kernel produces bit-identical cells.
//
// Reference semantics (epignatelli/cardiax):
//   derivative along an axis   cardiax/solve.py:225-254  (g_head / g_central / g_tail)
//   reaction + gates           cardiax/solve.py:34-42,57-59
//   stimulus override          cardiax/solve.py:44-46,257-271
//   Euler update               cardiax/solve.py:68-70
// The reference divides by dx and by the time constants; here each division is a multiply by
// the float32 reciprocal computed once on the host, and sums of coefficient products are fused
// multiply-adds in the reference's left-to-right order.  Both change results only at the level
// of the last bit of each operation (the parity tests bound the accumulated effect).
#pragma once
#include <cstdint>

namespace fk {

// Stencil coefficients of cardiax/solve.py:232-249, rounded to float32.
constexpr float C_HEAD0 = (float)(-11.0 / 6.0);
constexpr float C_THREE = 3.0f;
constexpr float C_3_2 = 1.5f;
constexpr float C_1_3 = (float)(1.0 / 3.0);
constexpr float C_1_12 = (float)(1.0 / 12.0);
constexpr float C_2_3 = (float)(2.0 / 3.0);
constexpr float C_TAIL0 = (float)(-1.0 / 3.0);
constexpr float C_TAIL3 = (float)(11.0 / 6.0);

// Interior 4th-order derivative on samples at offsets -2, -1, +1, +2 (un-scaled).
__device__ __forceinline__ float g_central(float m2, float m1, float p1, float p2) {
    float s = C_1_12 * m2;
    s = fmaf(-C_2_3, m1, s);
    s = fmaf(C_2_3, p1, s);
    return fmaf(-C_1_12, p2, s);
}
// 3rd-order one-sided derivative on samples at offsets 0, +1, +2, +3 (the first two rows).
__device__ __forceinline__ float g_head(float a0, float a1, float a2, float a3) {
    float s = C_HEAD0 * a0;
    s = fmaf(C_THREE, a1, s);
    s = fmaf(-C_3_2, a2, s);
    return fmaf(C_1_3, a3, s);
}
// 3rd-order one-sided derivative on samples at offsets -3, -2, -1, 0 (the last two rows).
__device__ __forceinline__ float g_tail(float a0, float a1, float a2, float a3) {
    float s = C_TAIL0 * a0;
    s = fmaf(C_3_2, a1, s);
    s = fmaf(-C_THREE, a2, s);
    return fmaf(C_TAIL3, a3, s);
}

__device__ __forceinline__ float4 g_central4(float4 m2, float4 m1, float4 p1, float4 p2) {
    return make_float4(g_central(m2.x, m1.x, p1.x, p2.x), g_central(m2.y, m1.y, p1.y, p2.y),
                       g_central(m2.z, m1.z, p1.z, p2.z), g_central(m2.w, m1.w, p1.w, p2.w));
}
__device__ __forceinline__ float4 mul4(float4 a, float s) {
    return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}

// Model constants of one tissue, prepared on the host from the 14 reference parameters
// (cardiax/params.py:4-18).  r_* are float32 reciprocals of the corresponding divisors.
struct Model {
    float V_c, V_v, V_csi, k;
    float r_tau_d, r_tau_0, inv_tau_r, r_2tau_si, r_Cm;
    float r_tau_v1m, r_tau_v2m, r_tau_vp, r_tau_wm, r_tau_wp;
    float pad0, pad1;
};

// One stimulus (cardiax/stimulus.py:13-21).  Protocol values are float32 as in the reference's
// loop (its step index is a float32); a stimulus is either a rectangle of constant amplitude
// (field == nullptr) or a dense field with the grid's pitch.
struct Stim {
    float start, duration, period, amplitude;
    int32_t r0, r1, c0, c1;
    const float *field;
    int64_t field_plane;  // element offset between tissues' fields in batched use (0 otherwise)
};

constexpr int kMaxStim = 8;

// Floor-mod protocol test of cardiax/solve.py:262-267 in float32.
__device__ __forceinline__ bool stim_active(const Stim &s, float t) {
    if (!(t >= s.start)) return false;
    float a = (s.start - t) + 1.0f;
    float m = fmodf(a, s.period);
    if (m != 0.0f && ((s.period < 0.0f) != (m < 0.0f))) m += s.period;
    return m < s.duration;
}

// 1 + tanh(x), through the identity 1 + tanh(x) = 2 / (1 + exp(-2x)), with the hardware
// base-2 exponential and reciprocal approximations (ex2.approx, rcp.approx: a few ulp).  The
// identity has no cancellation for x << 0 (the resting state, x ~ -8.5), where the reference
// computes 1 + tanh(x) after rounding tanh to float32.  Saturates correctly: x -> -inf gives 0
// (exp overflows to +inf, rcp(+inf) = 0), x -> +inf gives 2.
__device__ __forceinline__ float one_plus_tanh(float x) {
    const float kM2Log2e = -2.8853900817779268f;  // -2 / ln(2)
    float e, r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x * kM2Log2e));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
    return 2.0f * r;
}

// Ionic model: gates, currents, gate derivatives (cardiax/solve.py:34-42,57-58).
struct Reaction {
    float dv, dw, j_ion;
};
__device__ __forceinline__ Reaction reaction(float u, float v, float w, const Model &m) {
    const bool p = u >= m.V_c;
    const bool q = u >= m.V_v;
    // both sides of every gate are evaluated, then selected (no branches)
    // j_fi = -v p (u - V_c)(1 - u) / tau_d  (zero when the gate is closed)
    const float jfi_on = ((-v * (u - m.V_c)) * (1.0f - u)) * m.r_tau_d;
    const float j_fi = p ? jfi_on : 0.0f;
    // j_so = u (1 - p) / tau_0 + p / tau_r
    const float jso_off = u * m.r_tau_0;
    const float j_so = p ? m.inv_tau_r : jso_off;
    // j_si = -w (1 + tanh(k (u - V_csi))) / (2 tau_si)
    const float j_si = -(w * one_plus_tanh(m.k * (u - m.V_csi))) * m.r_2tau_si;
    Reaction r;
    r.j_ion = -((j_fi + j_so) + j_si) * m.r_Cm;
    const float r_tvm = q ? m.r_tau_v2m : m.r_tau_v1m;
    const float dv_on = -(v * m.r_tau_vp), dv_off = (1.0f - v) * r_tvm;
    const float dw_on = -(w * m.r_tau_wp), dw_off = (1.0f - w) * m.r_tau_wm;
    r.dv = p ? dv_on : dv_off;
    r.dw = p ? dw_on : dw_off;
    return r;
}

// del(u) = D (u_xx + u_yy) + D_x u_x + D_y u_y  (cardiax/solve.py:55)
__device__ __forceinline__ float diffusion(float d, float dx_, float dy_, float ux, float uy,
                                           float uxx, float uyy) {
    return fmaf(dy_, uy, fmaf(dx_, ux, d * (uxx + uyy)));
}



}  // namespace fk
