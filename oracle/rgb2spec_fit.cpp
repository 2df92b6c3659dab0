// rgb2spec_fit.cpp — TEST INFRASTRUCTURE ONLY (the oracle). CPU fit of an sRGB -> sigmoid-polynomial spectrum
// table in vkrt's layout (src/core/scene/rgb2spec.c:17-59: res z-scale floats, then 3*res^3*3 coefficients read
// by utility/rgb2spec.slang:33-81). Method: Jakob & Hanika 2019, "A Low-Dimensional Function Space for Efficient
// Spectral Upsampling": per cell, Gauss-Newton on the CIELAB residual of the reflected colour with a finite-
// difference Jacobian, warm-started from the neighbouring brightness level; coefficients live in normalised
// wavelength t = (lambda - 360) / 470 during the fit and are converted to nanometres on output.
// The colour-matching functions are the CIE 1931 analytic fits vkrt itself integrates with
// (utility/spectral.slang:66-87) under illuminant E, and XYZ -> linear sRGB is vkrt's output transform
// (Bradford E -> D65 then the sRGB matrix, utility/spectral.slang:14-20,89-97), so a spectrum fitted here
// reproduces its RGB exactly through vkrt's own display path. The device generator in the product is
// validated against this fit.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <atomic>
#include <vector>

#include "oracle.h"

namespace {

constexpr int kFine = 283;  // 94 intervals of 5 nm split in three (composite Simpson 3/8)
constexpr double kLmin = 360.0, kLmax = 830.0;

double cieX(double l) {
    double t1 = (l - 442.0) * (l < 442.0 ? 0.0624 : 0.0374);
    double t2 = (l - 599.8) * (l < 599.8 ? 0.0264 : 0.0323);
    double t3 = (l - 501.1) * (l < 501.1 ? 0.0490 : 0.0382);
    return std::max(0.0, 0.362 * std::exp(-0.5 * t1 * t1) + 1.056 * std::exp(-0.5 * t2 * t2) - 0.065 * std::exp(-0.5 * t3 * t3));
}
double cieY(double l) {
    double t1 = (l - 568.8) * (l < 568.8 ? 0.0213 : 0.0247);
    double t2 = (l - 530.9) * (l < 530.9 ? 0.0613 : 0.0322);
    return std::max(0.0, 0.821 * std::exp(-0.5 * t1 * t1) + 0.286 * std::exp(-0.5 * t2 * t2));
}
double cieZ(double l) {
    double t1 = (l - 437.0) * (l < 437.0 ? 0.0845 : 0.0278);
    double t2 = (l - 459.0) * (l < 459.0 ? 0.0385 : 0.0725);
    return std::max(0.0, 1.217 * std::exp(-0.5 * t1 * t1) + 0.681 * std::exp(-0.5 * t2 * t2));
}

void mul33(const double a[9], const double b[9], double o[9]) {
    double r[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] + a[i * 3 + 2] * b[2 * 3 + j];
    std::memcpy(o, r, sizeof(r));
}

bool inv33(const double m[9], double o[9]) {
    double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (det == 0.0) return false;
    double id = 1.0 / det;
    o[0] = (m[4] * m[8] - m[5] * m[7]) * id;
    o[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[3] = (m[5] * m[6] - m[3] * m[8]) * id;
    o[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[6] = (m[3] * m[7] - m[4] * m[6]) * id;
    o[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return true;
}

struct Tables {
    double t[kFine];        // normalised wavelength of each fine sample
    double rgbW[3][kFine];  // quadrature weight x (XYZ -> sRGB of the CMF sample)
    double xyzToRgb[9], rgbToXyz[9];
    double white[3];        // XYZ of the equal-energy spectrum
};

Tables makeTables() {
    Tables T;
    const double xyz2srgb[9] = {3.2404542, -1.5371385, -0.4985314, -0.9692660, 1.8760108, 0.0415560,
                                0.0556434, -0.2040259, 1.0572252};
    const double brad[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296};
    const double bradInv[9] = {0.9869929, -0.1470543, 0.1599627, 0.4323053, 0.5183603,
                               0.0492912, -0.0085287, 0.0400428, 0.9684867};
    const double scale[9] = {0.9413344, 0, 0, 0, 1.0404175, 0, 0, 0, 1.0895327};
    double tmp[9];
    mul33(scale, brad, tmp);
    mul33(bradInv, tmp, tmp);
    mul33(xyz2srgb, tmp, T.xyzToRgb);
    inv33(T.xyzToRgb, T.rgbToXyz);
    double h = (kLmax - kLmin) / double(kFine - 1);
    double ySum = 0.0;
    double w[kFine];
    for (int i = 0; i < kFine; ++i) {
        double wt = 3.0 * h / 8.0;
        if (i == 0 || i == kFine - 1) wt *= 1.0;
        else if ((i - 1) % 3 == 2) wt *= 2.0;
        else wt *= 3.0;
        w[i] = wt;
        ySum += wt * cieY(kLmin + h * i);
    }
    T.white[0] = T.white[1] = T.white[2] = 0.0;
    for (int i = 0; i < kFine; ++i) {
        double l = kLmin + h * i;
        T.t[i] = (l - kLmin) / (kLmax - kLmin);
        double xyz[3] = {cieX(l) * w[i] / ySum, cieY(l) * w[i] / ySum, cieZ(l) * w[i] / ySum};
        for (int k = 0; k < 3; ++k) {
            T.rgbW[k][i] = T.xyzToRgb[k * 3 + 0] * xyz[0] + T.xyzToRgb[k * 3 + 1] * xyz[1] + T.xyzToRgb[k * 3 + 2] * xyz[2];
            T.white[k] += xyz[k];
        }
    }
    return T;
}

double labF(double t) {
    const double d = 6.0 / 29.0;
    return t > d * d * d ? std::cbrt(t) : t / (3.0 * d * d) + 4.0 / 29.0;
}

void toLab(const Tables& T, const double rgb[3], double lab[3]) {
    double xyz[3];
    for (int k = 0; k < 3; ++k) xyz[k] = T.rgbToXyz[k * 3 + 0] * rgb[0] + T.rgbToXyz[k * 3 + 1] * rgb[1] + T.rgbToXyz[k * 3 + 2] * rgb[2];
    double fx = labF(xyz[0] / T.white[0]), fy = labF(xyz[1] / T.white[1]), fz = labF(xyz[2] / T.white[2]);
    lab[0] = 116.0 * fy - 16.0;
    lab[1] = 500.0 * (fx - fy);
    lab[2] = 200.0 * (fy - fz);
}

void reflectedRgb(const Tables& T, const double c[3], double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    for (int i = 0; i < kFine; ++i) {
        double x = (c[0] * T.t[i] + c[1]) * T.t[i] + c[2];
        double s = 0.5 * x / std::sqrt(1.0 + x * x) + 0.5;
        for (int k = 0; k < 3; ++k) out[k] += T.rgbW[k][i] * s;
    }
}

void residual(const Tables& T, const double c[3], const double target[3], double r[3]) {
    double got[3], a[3], b[3];
    reflectedRgb(T, c, got);
    toLab(T, target, a);
    toLab(T, got, b);
    for (int k = 0; k < 3; ++k) r[k] = a[k] - b[k];
}

double norm3(const double r[3]) { return std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]); }

// Gauss-Newton with a halving line search on the residual norm (the undamped step of the paper diverges when the
// warm start is far from the new target)
void gaussNewton(const Tables& T, const double target[3], double c[3]) {
    for (int it = 0; it < 15; ++it) {
        double r[3];
        residual(T, c, target, r);
        double rn0 = norm3(r);
        if (rn0 < 1e-6) break;
        double J[9];
        for (int j = 0; j < 3; ++j) {
            double c0[3] = {c[0], c[1], c[2]}, c1[3] = {c[0], c[1], c[2]};
            c0[j] -= 1e-4;
            c1[j] += 1e-4;
            double r0[3], r1[3];
            residual(T, c0, target, r0);
            residual(T, c1, target, r1);
            for (int i = 0; i < 3; ++i) J[i * 3 + j] = (r1[i] - r0[i]) / 2e-4;
        }
        double Ji[9];
        if (!inv33(J, Ji)) break;
        double dx[3];
        for (int i = 0; i < 3; ++i) dx[i] = Ji[i * 3 + 0] * r[0] + Ji[i * 3 + 1] * r[1] + Ji[i * 3 + 2] * r[2];
        double step = 1.0;
        double trial[3];
        for (int ls = 0; ls < 12; ++ls, step *= 0.5) {
            for (int i = 0; i < 3; ++i) trial[i] = c[i] - step * dx[i];
            double m = std::max(std::fabs(trial[0]), std::max(std::fabs(trial[1]), std::fabs(trial[2])));
            if (m > 200.0)
                for (int i = 0; i < 3; ++i) trial[i] *= 200.0 / m;
            double rt[3];
            residual(T, trial, target, rt);
            if (norm3(rt) < rn0) break;
        }
        for (int i = 0; i < 3; ++i) c[i] = trial[i];
    }
}

// walks the target from brightness b0 to b1 in steps of at most 0.02 so each solve starts close to its root
void solveFrom(const Tables& T, uint32_t l, double x, double y, double b0, double b1, double c[3]) {
    int steps = std::max(1, int(std::ceil(std::fabs(b1 - b0) / 0.02)));
    for (int s = 1; s <= steps; ++s) {
        double b = b0 + (b1 - b0) * double(s) / double(steps);
        double rgb[3];
        rgb[l] = b;
        rgb[(l + 1) % 3] = x * b;
        rgb[(l + 2) % 3] = y * b;
        gaussNewton(T, rgb, c);
    }
}

double smoothstep(double x) { return x * x * (3.0 - 2.0 * x); }

}  // namespace

extern "C" int32_t oracle_rgb2spec_generate(uint32_t res, float* out, uint32_t floatCount, uint32_t threads) {
    if (res < 3 || !out) return -1;
    size_t need = size_t(res) + size_t(3) * res * res * res * 3;
    if (floatCount < need) return -1;
    Tables T = makeTables();
    std::vector<double> scale(res);
    for (uint32_t k = 0; k < res; ++k) scale[k] = smoothstep(smoothstep(double(k) / double(res - 1)));
    for (uint32_t k = 0; k < res; ++k) out[k] = float(scale[k]);
    float* data = out + res;
    const double c0 = kLmin, c1 = 1.0 / (kLmax - kLmin);
    uint32_t jobs = 3 * res * res;
    std::atomic<uint32_t> next(0);
    unsigned nt = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
    auto work = [&]() {
        for (;;) {
            uint32_t job = next.fetch_add(1);
            if (job >= jobs) break;
            uint32_t l = job / (res * res), j = (job / res) % res, i = job % res;
            double x = double(i) / double(res - 1), y = double(j) / double(res - 1);
            uint32_t start = res / 5;
            for (int pass = 0; pass < 2; ++pass) {
                double c[3] = {0.0, 0.0, 0.0};
                int k = int(start), stop = pass == 0 ? int(res) : -1, step = pass == 0 ? 1 : -1;
                double bPrev = scale[start];
                solveFrom(T, l, x, y, bPrev, bPrev, c);
                for (; k != stop; k += step) {
                    double b = scale[uint32_t(k)];
                    solveFrom(T, l, x, y, bPrev, b, c);
                    bPrev = b;
                    double A = c[0], B = c[1], C = c[2];
                    size_t idx = ((((size_t(l) * res + uint32_t(k)) * res + j) * res + i) * 3);
                    data[idx + 0] = float(A * c1 * c1);
                    data[idx + 1] = float(B * c1 - 2.0 * A * c0 * c1 * c1);
                    data[idx + 2] = float(C - B * c0 * c1 + A * c0 * c0 * c1 * c1);
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    return 0;
}
