/*
 * iir_oracle.c — CPU oracle for the cascaded-biquad filtering path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the library links or calls this file; only tests/,
 * __graft_entry__.smoke() and the CPU-baseline / reference legs of bench.py load it, and only
 * as the reference output results are compared with (or as the timed CPU implementation of the
 * reference's golden path).
 *
 * Restated algorithms (own code, from the reference's behaviour):
 *   oracle_sosfilt_f64   — the reference's golden output: tools/ref_generate.py:89 calls
 *                          scipy.signal.sosfilt on float64 copies of the float32 input and the
 *                          float32-rounded normalised sections. scipy (un-vendored, unpinned in
 *                          the reference; 1.18.1 here) evaluates each section in transposed
 *                          direct form II, sample-major with the sections innermost
 *                          (scipy/signal/_sosfilt.pyx). Restated here in FP64 with the same
 *                          operation order.
 *   oracle_direct_f32    — float32 sequential direct form of order k, every product and sum
 *                          rounded to float32 in the order of tools/plr_emulator.py:185-202
 *                          (t = x[n]; t += b_j x[n-1-j]; y = t; y += a_j y[n-1-j]); it predicts
 *                          the PLR accuracy verdict (plr_emulator.py:228-248).
 *   oracle_cascade_f32   — float32 sequential cascade in the kernels' form
 *                          y = x + b1 x1 + b2 x2 + a1 y1 + a2 y2 with fmaf, section by section
 *                          (include/ph_kernels.cuh:157-161 coefficient convention).
 *   oracle_merge_sections— FP64 product of normalised sections into one direct-form pair,
 *                          the PLR route (tools/ref_generate.py:74-81 designs it with butter(ba)).
 *   oracle_normalise_sos — b0/a0 normalisation and the removed gain
 *                          (tools/ref_generate.py:62-67).
 */
#include <math.h>
#include <stddef.h>
#include <string.h>

/* y[n] = sosfilt(sos, x) in FP64, zero initial state. sos rows: b0 b1 b2 a0 a1 a2 (a0 may be != 1:
 * rows are divided by a0 first, which scipy requires to already hold). */
void oracle_sosfilt_f64(const double* x, long long n, const double* sos, int n_sections, double* y) {
    double z[2 * 64];
    double c[6 * 64];
    int s;
    long long i;
    if (n_sections > 64) return;
    for (s = 0; s < n_sections; ++s) {
        const double a0 = sos[6 * s + 3];
        int k;
        for (k = 0; k < 6; ++k) c[6 * s + k] = sos[6 * s + k] / a0;
        z[2 * s] = 0.0;
        z[2 * s + 1] = 0.0;
    }
    for (i = 0; i < n; ++i) {
        double xc = x[i];
        for (s = 0; s < n_sections; ++s) {
            const double* q = c + 6 * s;
            const double xn = q[0] * xc + z[2 * s];
            z[2 * s] = q[1] * xc - q[4] * xn + z[2 * s + 1];
            z[2 * s + 1] = q[2] * xc - q[5] * xn;
            xc = xn;
        }
        y[i] = xc;
    }
}

/* float32 sequential direct form: b[k], a[k] as float32, recurrence sign y[n] += a_j y[n-1-j]. */
void oracle_direct_f32(const float* x, long long n, const float* b, const float* a, int k, float* y) {
    float xh[32], yh[32];
    long long i;
    int j;
    if (k > 32) return;
    for (j = 0; j < k; ++j) {
        xh[j] = 0.f;
        yh[j] = 0.f;
    }
    for (i = 0; i < n; ++i) {
        volatile float t = x[i];
        volatile float o;
        for (j = 0; j < k; ++j) {
            volatile float p = b[j] * xh[j];
            t = t + p;
        }
        o = t;
        for (j = 0; j < k; ++j) {
            volatile float p = a[j] * yh[j];
            o = o + p;
        }
        for (j = k - 1; j > 0; --j) {
            xh[j] = xh[j - 1];
            yh[j] = yh[j - 1];
        }
        xh[0] = x[i];
        yh[0] = o;
        y[i] = o;
    }
}

/* float32 sequential cascade, normalised float32 coefficients coef[4*s..] = {b1, b2, a1, a2}
 * (a1 = -sos[4], a2 = -sos[5]); input already multiplied by the gain. */
void oracle_cascade_f32(const float* x, long long n, const float* coef, int n_sections, float* y) {
    long long i;
    int s;
    for (i = 0; i < n; ++i) y[i] = x[i];
    for (s = 0; s < n_sections; ++s) {
        const float b1 = coef[4 * s], b2 = coef[4 * s + 1], a1 = coef[4 * s + 2], a2 = coef[4 * s + 3];
        float x1 = 0.f, x2 = 0.f, y1 = 0.f, y2 = 0.f;
        for (i = 0; i < n; ++i) {
            const float xv = y[i];
            const float w = fmaf(b2, x2, fmaf(b1, x1, xv));
            const float v = fmaf(a1, y1, fmaf(a2, y2, w));
            x2 = x1;
            x1 = xv;
            y2 = y1;
            y1 = v;
            y[i] = v;
        }
    }
}

/* Normalises rows to b0 = a0 = 1 in FP64. out rows keep the scipy layout {1, b1, b2, 1, a1, a2}.
 * Returns the removed gain prod(b0 / a0). */
double oracle_normalise_sos(const double* sos, int n_sections, double* out) {
    double g = 1.0;
    int s;
    for (s = 0; s < n_sections; ++s) {
        const double b0 = sos[6 * s], a0 = sos[6 * s + 3];
        g *= b0 / a0;
        out[6 * s + 0] = 1.0;
        out[6 * s + 1] = sos[6 * s + 1] / b0;
        out[6 * s + 2] = sos[6 * s + 2] / b0;
        out[6 * s + 3] = 1.0;
        out[6 * s + 4] = sos[6 * s + 4] / a0;
        out[6 * s + 5] = sos[6 * s + 5] / a0;
    }
    return g;
}

/* Product of normalised sections (rows {1,b1,b2,1,a1,a2}) as one direct form of order 2K:
 * b_out[j] = taps past b0 = 1, a_out[j] = recurrence taps (y[n] += a_out[j] y[n-1-j]). */
void oracle_merge_sections(const double* sos_norm, int n_sections, double* b_out, double* a_out) {
    double bp[2 * 64 + 1], ap[2 * 64 + 1], nb[2 * 64 + 1], na[2 * 64 + 1];
    int len = 1, s, i, j;
    if (n_sections > 64) return;
    bp[0] = 1.0;
    ap[0] = 1.0;
    for (s = 0; s < n_sections; ++s) {
        const double bs[3] = {1.0, sos_norm[6 * s + 1], sos_norm[6 * s + 2]};
        const double as[3] = {1.0, sos_norm[6 * s + 4], sos_norm[6 * s + 5]};
        for (i = 0; i < len + 2; ++i) {
            nb[i] = 0.0;
            na[i] = 0.0;
        }
        for (i = 0; i < len; ++i)
            for (j = 0; j < 3; ++j) {
                nb[i + j] += bp[i] * bs[j];
                na[i + j] += ap[i] * as[j];
            }
        len += 2;
        memcpy(bp, nb, sizeof(double) * len);
        memcpy(ap, na, sizeof(double) * len);
    }
    for (i = 1; i < len; ++i) {
        b_out[i - 1] = bp[i];
        a_out[i - 1] = -ap[i];
    }
}
