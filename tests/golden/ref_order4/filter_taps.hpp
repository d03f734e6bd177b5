// Auto-generated by ref_generate.py — DO NOT EDIT.
// Butterworth lowpass, order 4, cutoff 0.2 x Nyquist.
// Sections are normalized to b0 == 1; FILTER_GAIN is the removed
// cascade gain and must be pre-applied to the input signal.
#pragma once

#define FILTER_N_SECTIONS 2
static const double FILTER_GAIN = 0.004824343357716228;
static const double INPUT_FS    = 1000.0;
static const double INPUT_FREQ  = 120.0;

static const float FILTER_SOS[2][6] = {
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.048599601e+00f, 2.961403430e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.320913434e+00f, 6.327387691e-01f}
};

// Direct-form realization of the SAME transfer function (PLR lane).
// b0-normalized (implicit b0 == 1, gain removed = FILTER_GAIN);
// A uses the recurrence sign convention y[n] += A[j] * y[n-j-1].
#define PLR_FILTER_ORDER 4
static const double PLR_FILTER_B[4] = {
    4.0,
    6.0,
    4.0,
    1.0
};
static const double PLR_FILTER_A[4] = {
    2.369513007182038,
    -2.313988414415881,
    1.054665405878568,
    -0.18737949236818502
};
