// log10 of a single evaluated in double and rounded once, identical on the
// host and the device: the binary exponent is split off (mantissa in
// [sqrt(1/2), sqrt(2))), ln of the mantissa from the atanh series
// ln m = 2 (s + s^3/3 + ... + s^23/23), s = (m - 1) / (m + 1).
#pragma once

#include <cmath>

namespace tg {

__host__ __device__ inline float log10_single(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int e;
    double m = frexp((double)x, &e);
    if (m < 0.70710678118654752) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double t = 1.0 / 23.0;
    for (int k = 21; k >= 1; k -= 2) t = 1.0 / k + s2 * t;
    const double ln = 2.0 * s * t + (double)e * 0.69314718055994530942;
    return (float)(ln / 2.30258509299404568402);
}

// slice layout and particle weights of a spectrum writer
struct SpecGrid {
    int mxmin, mymin, nxb, nyb, gambins;
    float dxslice, dyslice;
    int ind_filter;    // only particles with ind > 0 count (save_spectrum_2d)
    int split;         // weight splitratio^(1 - splitlev) * ch (save_spectrum)
    float wsplit[32];  // splitratio^(1 - s) for splitlev s in [0, 32)
};
// save_spectrum_2d (code/output.F90:828-852): slices of 30 cells

inline SpecGrid spec_grid(int mx, int my, int ng, int gambins) {
    SpecGrid s;
    const int mxmin = (int)((float)(mx - ng) * 0.5f) - 1200 + (ng / 2 + 1);
    const int mxmax = (int)((float)(mx - ng) * 0.5f) + 400 + (ng / 2 + 1);
    const int mymin = ng / 2 + 1, mymax = my - ng / 2;
    s.mxmin = mxmin;
    s.mymin = mymin;
    s.nxb = (mxmax - mxmin) / 30 > 1 ? (mxmax - mxmin) / 30 : 1;
    s.nyb = (mymax - mymin) / 30 > 1 ? (mymax - mymin) / 30 : 1;
    s.gambins = gambins;
    s.dxslice = 1.0f * (float)(mxmax - mxmin) / (float)s.nxb;
    s.dyslice = 1.0f * (float)(mymax - mymin) / (float)s.nyb;
    s.ind_filter = 1;
    s.split = 0;
    for (int k = 0; k < 32; k++) s.wsplit[k] = 1.0f;
    return s;
}
// save_spectrum (code/output.F90:424-437): x slices of about 100 cells over
// [3, mx0 - 2], one slice in y; weights splitratio^(1 - splitlev) ch with
// the legacy splitratio = 10 (code/particles.F90:336), powers from the
// host's powf as the reference's real**real
inline SpecGrid spec_grid_x(int mx, int gambins) {
    SpecGrid s;
    const int mxmin = 3, mxmax = mx - 2;
    s.mxmin = mxmin;
    s.mymin = 0;
    s.nxb = (mxmax - mxmin) / 100 > 1 ? (mxmax - mxmin) / 100 : 1;
    s.nyb = 1;
    s.gambins = gambins;
    s.dxslice = 1.0f * (float)(mxmax - mxmin) / (float)s.nxb;
    s.dyslice = INFINITY;  // every y in the one slice
    s.ind_filter = 0;
    s.split = 1;
    for (int k = 0; k < 32; k++) s.wsplit[k] = powf(10.0f, 1.0f - (float)k);
    return s;
}

}  // namespace tg
