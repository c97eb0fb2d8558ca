/*
 * CPU oracle for the Fenton-Karma Euler stepper -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's forward path (epignatelli/cardiax), used by the
 * tests as a checker for large grids and by bench.py as the timed CPU baseline ("port").  It is
 * never linked into the product library.
 *
 * It follows cardiax/solve.py in the reference's evaluation order (so that float32 results round
 * the same way; compile with -ffp-contract=off):
 *   step            solve.py:26-65   -> fko_step_*            (edge pad, reaction, stimulus,
 *                                                               4th-order diffusion)
 *   step_euler      solve.py:68-70   -> Euler update inside fko_step_*
 *   _forward_euler  solve.py:92-100  -> fko_forward_euler_*
 *   gradient        solve.py:225-254 -> grad_at()
 *   stimulate       solve.py:257-271 -> stim_active() + the overwrite loop
 * The only operation whose last bit may differ from the NumPy oracle is tanh (libm vs NumPy).
 *
 * Parallelism: rows are split over OpenMP threads (the NumPy oracle is single-threaded).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double start, duration, period; /* protocol in steps, cardiax/stimulus.py:13-16 */
    const void *field;              /* dense H*W field of the working type            */
} fko_stim;

#define DEFINE_FK(T, SUF, TANH, FMOD)                                                          \
    /* padded-array derivative (solve.py:225-254) at padded index k of a length-L line */      \
    static inline T grad_at_##SUF(const T *P, long stride, long k, long L) {                  \
        const T c116 = (T)(-11.0 / 6.0), c3 = (T)3.0, c32 = (T)(3.0 / 2.0),                   \
                c13 = (T)(1.0 / 3.0), c112 = (T)(1.0 / 12.0), c23 = (T)(2.0 / 3.0),           \
                cm13 = (T)(-1.0 / 3.0), c116p = (T)(11.0 / 6.0);                              \
        if (k < 2) {                                                                           \
            const T *p = P + k * stride;                                                       \
            return ((c116 * p[0] + c3 * p[stride]) - c32 * p[2 * stride]) + c13 * p[3 * stride]; \
        }                                                                                      \
        if (k > L - 3) {                                                                       \
            const T *p = P + (k - 3) * stride;                                                 \
            return ((cm13 * p[0] + c32 * p[stride]) - c3 * p[2 * stride]) + c116p * p[3 * stride]; \
        }                                                                                      \
        const T *p = P + (k - 2) * stride;                                                     \
        return ((c112 * p[0] - c23 * p[stride]) + c23 * p[3 * stride]) - c112 * p[4 * stride]; \
    }                                                                                          \
    /* floor-mod protocol test (solve.py:262-267), in the working type */                      \
    static inline int stim_active_##SUF(T t, const fko_stim *s) {                              \
        T start = (T)s->start, dur = (T)s->duration, per = (T)s->period;                       \
        if (!(t >= start)) return 0;                                                           \
        T a = (start - t) + (T)1;                                                              \
        T m = FMOD(a, per);                                                                    \
        if (m != (T)0) {                                                                       \
            if ((per < (T)0) != (m < (T)0)) m += per;                                          \
        }                                                                                      \
        return m < dur;                                                                        \
    }                                                                                          \
    typedef struct {                                                                           \
        long H, W;                                                                             \
        T *pu;  /* (H+2)x(W+2) edge-padded u */                                                \
        T *ux;  /* (H+2)xW: d/dx of padded u, all padded rows, interior columns */             \
        T *uy;  /* Hx(W+2): d/dy of padded u, interior rows, all padded columns */             \
        T *dxD; /* HxW */                                                                      \
        T *dyD; /* HxW */                                                                      \
        T *pd;  /* (H+2)x(W+2) edge-padded D */                                                \
    } ws_##SUF;                                                                                \
    static void pad_edge_##SUF(const T *a, T *p, long H, long W) {                             \
        long PW = W + 2;                                                                       \
        for (long r = 0; r < H + 2; ++r) {                                                     \
            long i = r == 0 ? 0 : (r == H + 1 ? H - 1 : r - 1);                                \
            T *row = p + r * PW;                                                               \
            memcpy(row + 1, a + i * W, sizeof(T) * W);                                         \
            row[0] = a[i * W];                                                                 \
            row[W + 1] = a[i * W + W - 1];                                                     \
        }                                                                                      \
    }                                                                                          \
    static int step_##SUF(ws_##SUF *ws, const T *v, const T *w, const T *u, T *vn, T *wn,      \
                          T *un, const T *D, const double *prm, const fko_stim *st, int ns,    \
                          T t, T dt, T dx, int nthreads) {                                     \
        long H = ws->H, W = ws->W, PW = W + 2, L0 = H + 2, L1 = W + 2;                         \
        (void)nthreads;                                                                        \
        const T tvp = (T)prm[0], tv1m = (T)prm[1], tv2m = (T)prm[2], twp = (T)prm[3],          \
                twm = (T)prm[4], td = (T)prm[5], t0 = (T)prm[6], tr = (T)prm[7],               \
                tsi = (T)prm[8], kk = (T)prm[9], vcsi = (T)prm[10], vc = (T)prm[11],           \
                vv = (T)prm[12], cm = (T)prm[13];                                              \
        const T one = (T)1, two_tsi = (T)2 * tsi;                                              \
        int act[64];                                                                           \
        if (ns > 64) return -1;                                                                \
        for (int s = 0; s < ns; ++s) act[s] = stim_active_##SUF(t, &st[s]);                    \
        pad_edge_##SUF(u, ws->pu, H, W);                                                       \
        _Pragma("omp parallel for num_threads(nthreads) schedule(static)")                     \
        for (long r = 0; r < L0; ++r)                                                          \
            for (long j = 0; j < W; ++j)                                                       \
                ws->ux[r * W + j] = grad_at_##SUF(ws->pu + j + 1, PW, r, L0) / dx;             \
        _Pragma("omp parallel for num_threads(nthreads) schedule(static)")                     \
        for (long i = 0; i < H; ++i)                                                           \
            for (long c = 0; c < L1; ++c)                                                      \
                ws->uy[i * L1 + c] = grad_at_##SUF(ws->pu + (i + 1) * PW, 1, c, L1) / dx;      \
        _Pragma("omp parallel for num_threads(nthreads) schedule(static)")                     \
        for (long i = 0; i < H; ++i) {                                                         \
            for (long j = 0; j < W; ++j) {                                                     \
                long c = i * W + j;                                                            \
                T uu = u[c], vv_ = v[c], ww = w[c], dd = D[c];                                 \
                T p = uu >= vc ? one : (T)0;                                                   \
                T q = uu >= vv ? one : (T)0;                                                   \
                T tvm = (one - q) * tv1m + q * tv2m;                                           \
                T j_fi = -vv_ * p * (uu - vc) * (one - uu) / td;                               \
                T j_so = (uu * (one - p) / t0) + (p / tr);                                     \
                T j_si = -(ww * (one + TANH(kk * (uu - vcsi)))) / two_tsi;                     \
                T j_ion = -(j_fi + j_so + j_si) / cm;                                          \
                T acc = (T)0;                                                                  \
                for (int s = 0; s < ns; ++s)                                                   \
                    if (act[s]) {                                                              \
                        T f = ((const T *)st[s].field)[c];                                     \
                        if (f != (T)0) acc = f;                                                \
                    }                                                                          \
                if (acc != (T)0) j_ion = acc;                                                  \
                T uxx = grad_at_##SUF(ws->ux + j, W, i + 1, L0) / dx;                          \
                T uyy = grad_at_##SUF(ws->uy + i * L1, 1, j + 1, L1) / dx;                     \
                T ux = ws->ux[(i + 1) * W + j], uy = ws->uy[i * L1 + j + 1];                   \
                T del = dd * (uxx + uyy) + (ws->dxD[c] * ux) + (ws->dyD[c] * uy);              \
                T dv = ((one - p) * (one - vv_) / tvm) - ((p * vv_) / tvp);                    \
                T dw = ((one - p) * (one - ww) / twm) - ((p * ww) / twp);                      \
                T du = del + j_ion;                                                            \
                vn[c] = vv_ + dv * dt;                                                         \
                wn[c] = ww + dw * dt;                                                          \
                un[c] = uu + du * dt;                                                          \
            }                                                                                  \
        }                                                                                      \
        return 0;                                                                              \
    }                                                                                          \
    int fko_forward_euler_##SUF(T *v, T *w, T *u, const T *D, long H, long W,                  \
                                const double *params, const fko_stim *stims, int n_stims,      \
                                long t0, long t1, double dt, double dx, int nthreads,          \
                                int *act_first, int *act_last, int *act_count,                 \
                                double threshold) {                                            \
        if (H < 3 || W < 3) return -2;                                                         \
        if (nthreads < 1) nthreads = 1;                                                        \
        ws_##SUF ws;                                                                           \
        ws.H = H; ws.W = W;                                                                    \
        size_t n = (size_t)H * W, np_ = (size_t)(H + 2) * (W + 2);                             \
        ws.pu = malloc(sizeof(T) * np_); ws.pd = malloc(sizeof(T) * np_);                      \
        ws.ux = malloc(sizeof(T) * (H + 2) * W); ws.uy = malloc(sizeof(T) * H * (W + 2));      \
        ws.dxD = malloc(sizeof(T) * n); ws.dyD = malloc(sizeof(T) * n);                        \
        T *bv = malloc(sizeof(T) * n), *bw = malloc(sizeof(T) * n), *bu = malloc(sizeof(T) * n); \
        int rc = 0;                                                                            \
        if (!ws.pu || !ws.pd || !ws.ux || !ws.uy || !ws.dxD || !ws.dyD || !bv || !bw || !bu) { \
            rc = -3; goto done;                                                                \
        }                                                                                      \
        T h = (T)dx, k = (T)dt;                                                                \
        /* D is constant in time: its derivatives are computed once (same values each step) */ \
        pad_edge_##SUF(D, ws.pd, H, W);                                                        \
        for (long i = 0; i < H; ++i)                                                           \
            for (long j = 0; j < W; ++j) {                                                     \
                ws.dxD[i * W + j] = grad_at_##SUF(ws.pd + j + 1, W + 2, i + 1, H + 2) / h;     \
                ws.dyD[i * W + j] = grad_at_##SUF(ws.pd + (i + 1) * (W + 2), 1, j + 1, W + 2) / h; \
            }                                                                                  \
        for (long s = t0; s < t1; ++s) {                                                       \
            rc = step_##SUF(&ws, v, w, u, bv, bw, bu, D, params, stims, n_stims, (T)s, k, h,   \
                            nthreads);                                                         \
            if (rc) goto done;                                                                 \
            if (act_last) {                                                                    \
                /* activation: upstroke of u through the threshold during step s -> s+1 */     \
                const T thr = (T)threshold;                                                    \
                for (size_t c = 0; c < n; ++c)                                                 \
                    if (u[c] < thr && bu[c] >= thr) {                                          \
                        act_last[c] = (int)(s + 1);                                            \
                        if (act_first[c] < 0) act_first[c] = (int)(s + 1);                     \
                        act_count[c] += 1;                                                     \
                    }                                                                          \
            }                                                                                  \
            memcpy(v, bv, sizeof(T) * n); memcpy(w, bw, sizeof(T) * n);                        \
            memcpy(u, bu, sizeof(T) * n);                                                      \
        }                                                                                      \
    done:                                                                                      \
        free(ws.pu); free(ws.pd); free(ws.ux); free(ws.uy); free(ws.dxD); free(ws.dyD);        \
        free(bv); free(bw); free(bu);                                                          \
        return rc;                                                                             \
    }

DEFINE_FK(float, f32, tanhf, fmodf)
DEFINE_FK(double, f64, tanh, fmod)

int fko_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
