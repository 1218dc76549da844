// Host-side FP64 construction of the Kaiser-Bessel lookup table and the
// pre-compensation (deapodization) vector.
#include <cmath>
#include <vector>

#include "gg_internal.h"

namespace gg {

// alpha for half-widths 1..5 (src/Matlab/utils/kernelAlpha.m:6).
static double kernel_alpha(int hw)
{
    static const double alphavals[5] = {5.5, 10.0, 10.2, 13.0, 17.0};
    if (hw < 1 || hw > 5) return 0.0;
    return alphavals[hw - 1];
}

// Modified Bessel function of the first kind, order 0, from its power series
// sum_k ((x/2)^k / k!)^2 (Abramowitz & Stegun 9.6.10).  For the arguments
// used here (x <= 20) the series reaches double precision well within 80 terms.
static double bessel_i0(double x)
{
    const double q = 0.25 * x * x;
    double term = 1.0, total = 1.0;
    for (int k = 1; k < 80; k++) {
        term *= q / ((double)k * (double)k);
        total += term;
        if (term < 1e-17 * total) break;
    }
    return total;
}

// Kaiser-Bessel window of half-width n (src/Matlab/utils/gridLibKaiser.m:5-15).
static double kaiser(double n, double alpha, double q)
{
    if (std::fabs(q) > n) return 0.0;
    const double r = std::sqrt(1.0 - (q / n) * (q / n));
    return bessel_i0(alpha * r) / bessel_i0(alpha);
}

// Points of MATLAB's a:d:b, evaluated from both ends like MATLAB's colon.
static std::vector<double> colon(double a, double d, double b)
{
    const int n = (int)std::floor((b - a) / d + 1e-10) + 1;
    std::vector<double> x(n);
    double last = a + (n - 1) * d;
    if (std::fabs(last - b) < 1e-9 * std::fmax(1.0, std::fabs(b))) last = b;
    for (int k = 0; k < n; k++) x[k] = (k < n / 2) ? a + k * d : last - (n - 1 - k) * d;
    return x;
}

// getKernelFiltTable(hw, size) (src/Matlab/utils/getKernelFiltTable.m:1-22):
// unit-integral window, edge value subtracted, last value forced to zero, then
// divided by the cube root of the sum over the (2hw+1)^3 integer taps.
void kb_table_f64(int hw, int size, double *out)
{
    const double alpha = kernel_alpha(hw);
    const double delta = 2.0 * hw / (size - 1);
    std::vector<double> x = colon(-hw, delta, hw);
    std::vector<double> w(size, 0.0);
    double s = 0.0;
    for (int i = 0; i < size && i < (int)x.size(); i++) {
        w[i] = kaiser(hw, alpha, x[i]);
        s += w[i] * delta;
    }
    for (int i = 0; i < size; i++) w[i] /= s;
    const double w0 = w[0];
    for (int i = 0; i < size; i++) w[i] -= w0;
    w[size - 1] = 0.0;
    // integer taps sit at 1-based index x*scale + center, x = -hw..hw
    const double center = (size + 1) / 2.0;
    const double scale = (center - 1) / hw;
    double ksum = 0.0;
    for (int t = -hw; t <= hw; t++) ksum += w[(int)std::lround(t * scale + center) - 1];
    const double denom = ksum * ksum * ksum; // sum of kron(kron(ker,ker'),ker)
    const double norm = std::cbrt(denom);
    for (int i = 0; i < size; i++) out[i] = w[i] / norm;
}

// getPreComp(M, hw) (src/Matlab/utils/getPreComp.m:1-28).  The window sampled
// at 1/4 voxel is symmetric, so real(fftshift(fft(fftshift(line)))) at
// frequency j is the cosine sum  P(j) = sum_m w_m cos(2 pi j m / (4M)),
// evaluated directly in FP64; out[t] = P(0) / P(t - M/2), t = 0..M-1.
void precomp_f64(int M, int hw, double *out)
{
    const int ovr = 4;
    const double alpha = kernel_alpha(hw);
    std::vector<double> x = colon(-hw, 1.0 / ovr, hw);
    const int nw = (int)x.size();
    std::vector<double> w(nw);
    for (int i = 0; i < nw; i++) w[i] = kaiser(hw, alpha, x[i]);
    const double w0 = w[0];
    for (int i = 0; i < nw; i++) w[i] -= w0;
    w[nw - 1] = 0.0;
    const int half = (nw - 1) / 2;
    const double L = (double)M * ovr;
    const double two_pi = 6.283185307179586476925286766559;
    auto P = [&](int j) {
        double acc = 0.0;
        for (int m = -half; m <= half; m++) acc += w[m + half] * std::cos(two_pi * (double)j * (double)m / L);
        return acc;
    };
    const double fc0 = P(0);
    for (int t = 0; t < M; t++) out[t] = fc0 / P(t - M / 2);
}

} // namespace gg
