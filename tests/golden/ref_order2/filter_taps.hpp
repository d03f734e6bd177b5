// Auto-generated by ref_generate.py — DO NOT EDIT.
// Butterworth lowpass, order 2, cutoff 0.2 x Nyquist.
// Sections are normalized to b0 == 1; FILTER_GAIN is the removed
// cascade gain and must be pre-applied to the input signal.
#pragma once

#define FILTER_N_SECTIONS 1
static const double FILTER_GAIN = 0.0674552738890719;
static const double INPUT_FS    = 1000.0;
static const double INPUT_FREQ  = 120.0;

static const float FILTER_SOS[1][6] = {
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.142980456e+00f, 4.128015935e-01f}
};

// Direct-form realization of the SAME transfer function (PLR lane).
// b0-normalized (implicit b0 == 1, gain removed = FILTER_GAIN);
// A uses the recurrence sign convention y[n] += A[j] * y[n-j-1].
#define PLR_FILTER_ORDER 2
static const double PLR_FILTER_B[2] = {
    2.0,
    1.0
};
static const double PLR_FILTER_A[2] = {
    1.1429805025399011,
    -0.41280159809618877
};
