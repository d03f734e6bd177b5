// Auto-generated by ref_generate.py — DO NOT EDIT.
// Butterworth lowpass, order 16, cutoff 0.2 x Nyquist.
// Sections are normalized to b0 == 1; FILTER_GAIN is the removed
// cascade gain and must be pre-applied to the input signal.
#pragma once

#define FILTER_N_SECTIONS 8
static const double FILTER_GAIN = 5.824202597102247e-10;
static const double INPUT_FS    = 1000.0;
static const double INPUT_FREQ  = 120.0;

static const float FILTER_SOS[8][6] = {
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.020870686e+00f, 2.618655562e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.035558105e+00f, 2.800201476e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.065631509e+00f, 3.171930611e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.112537026e+00f, 3.751714230e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.178563118e+00f, 4.567841291e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.266979337e+00f, 5.660725236e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.382196665e+00f, 7.084890008e-01f},
    {1.000000000e+00f, 2.000000000e+00f, 1.000000000e+00f, 1.000000000e+00f, -1.529892206e+00f, 8.910508156e-01f}
};

// Direct-form realization of the SAME transfer function (PLR lane).
// b0-normalized (implicit b0 == 1, gain removed = FILTER_GAIN);
// A uses the recurrence sign convention y[n] += A[j] * y[n-j-1].
#define PLR_FILTER_ORDER 16
static const double PLR_FILTER_B[16] = {
    16.0,
    120.0,
    560.0,
    1820.0,
    4368.0,
    8008.0,
    11440.0,
    12870.0,
    11440.0,
    8008.0,
    4368.0,
    1820.0,
    560.0,
    120.0,
    16.0,
    1.0
};
static const double PLR_FILTER_A[16] = {
    9.592228621725116,
    -43.99549555494624,
    127.79236096209958,
    -262.6519031741734,
    404.4528010368368,
    -482.1181305375409,
    453.3462745552862,
    -339.55542058661104,
    203.10054702757515,
    -96.62679661774769,
    36.159558249341785,
    -10.428634113566432,
    2.2397582300943677,
    -0.33768004150730047,
    0.03191819905531162,
    -0.0014244254154724845
};
