"""Generate ``es_table.h``: shape parameters of the exponential-of-semicircle
(ES) gridding kernel for each (oversampling factor, support width).

The ES kernel (Barnett, Magland & af Klinteberg 2019, SIAM J. Sci. Comput.
41(5), C479) on a support of W grid cells is

    phi(x) = exp(beta * (sqrt(1 - (2x/W)^2) - 1)),   |x| <= W/2.

Gridding onto a grid oversampled by sigma and dividing by the kernel's
Fourier transform phihat leaves an aliasing error at normalised frequency
nu (cycles per cell, |nu| <= 1/(2 sigma)) of

    e(nu) = sqrt(sum_{p != 0} phihat(nu + p)^2) / |phihat(nu)|.

For every (sigma, W) this script picks the beta that minimises
max_nu e(nu) and records that maximum.  The planner picks the smallest W
whose error, summed over the gridded dimensions, is below the requested
epsilon.  Run:  python gen_es_table.py > es_table.h
"""
import numpy as np
from numpy.polynomial.legendre import leggauss

SIGMAS = (1.25, 1.5, 1.75, 2.0)
WMIN, WMAX = 4, 16
XG, WG = leggauss(2500)


def phihat(nu, W, beta):
    x = XG * W / 2
    w = WG * W / 2
    ph = np.exp(beta * (np.sqrt(1.0 - (2 * x / W) ** 2) - 1.0))
    return (w * ph) @ np.cos(2 * np.pi * np.outer(x, nu))


def band_error(W, sigma, beta, naliases=24):
    nu = np.linspace(0.0, 0.5 / sigma, 41)
    main = phihat(nu, W, beta)
    al = np.zeros_like(nu)
    for p in range(1, naliases + 1):
        al += phihat(nu + p, W, beta) ** 2 + phihat(nu - p, W, beta) ** 2
    return float(np.max(np.sqrt(al) / np.abs(main)))


def best_beta(W, sigma):
    lo, hi = 1.2 * W, 2.8 * W
    grid = np.linspace(lo, hi, 33)
    errs = [band_error(W, sigma, b) for b in grid]
    i = int(np.argmin(errs))
    # golden-section refinement around the coarse minimum
    a, b = grid[max(i - 1, 0)], grid[min(i + 1, len(grid) - 1)]
    g = (np.sqrt(5) - 1) / 2
    c, d = b - g * (b - a), a + g * (b - a)
    fc, fd = band_error(W, sigma, c), band_error(W, sigma, d)
    for _ in range(18):
        if fc < fd:
            b, d, fd = d, c, fc
            c = b - g * (b - a)
            fc = band_error(W, sigma, c)
        else:
            a, c, fc = c, d, fd
            d = a + g * (b - a)
            fd = band_error(W, sigma, d)
    beta = (a + b) / 2
    return beta, band_error(W, sigma, beta)


def main():
    print("// Generated by gen_es_table.py -- ES kernel shape per (sigma, W).")
    print("// Columns: sigma, W, beta, max aliasing error per gridded dimension.")
    print("#pragma once")
    print("struct GbEsEntry { double sigma; int support; double beta; double error; };")
    print("static const GbEsEntry kGbEsTable[] = {")
    for s in SIGMAS:
        for W in range(WMIN, WMAX + 1):
            beta, err = best_beta(W, s)
            print(f"  {{{s:.2f}, {W:2d}, {beta:.10f}, {err:.4e}}},")
    print("};")
    print("static const int kGbEsTableSize = sizeof(kGbEsTable) / sizeof(kGbEsTable[0]);")


if __name__ == "__main__":
    main()
