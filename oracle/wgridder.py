"""FP64 numpy restatement of the w-stacking ES gridder (oracle; test
infrastructure only).

This restates, from the published method (Arras, Reinecke, Westermann &
Ensslin 2021, A&A 646, A58; ES kernel of Barnett et al. 2019), the
algorithm behind ``ducc0.wgridder.ms2dirty`` / ``dirty2ms`` that
``rascil/processing_components/imaging/ng.py:91-120,232-275`` calls, with
the same planning rules as the CUDA planner so that intermediate results
(plan geometry, uv-bucket keys) can be compared exactly:

* grid side ``ng = good_size(max(ceil(sigma n), 2W))``;
* u wraps modulo one image-Nyquist period: ``U = frac(u dx) ng``;
* first support cell ``p0 = ceil(U - W/2)``, offset ``du = U - p0``;
* w-planes spaced ``dw = 1/(2 sigma h)`` around the centre ``tc`` of the
  image's (n-1) range of half-width ``h``; visibilities are pre-rotated by
  ``exp(-2 pi i w tc)``;
* the grid carries a (-1)^(p+q) checkerboard so the image is the central
  block of the FFT output;
* correction ``1/(phihat(x'/ngx) phihat(y'/ngy) phihat(dw t') n)``.

Small cases only (vectorised numpy, O(nvis W^3) memory-light loops).
"""

import math
import os
import re

import numpy

from .dft import SPEED_OF_LIGHT

_TABLE_PATH = os.path.join(os.path.dirname(__file__), "..", "rascil_gb300",
                           "csrc", "es_table.h")


def es_table():
    """Parse the generated ES-kernel table: list of (sigma, W, beta, err)."""
    rows = []
    with open(_TABLE_PATH) as f:
        for line in f:
            m = re.match(r"\s*\{([0-9.]+),\s*(\d+),\s*([0-9.]+),\s*([0-9.e+-]+)\}", line)
            if m:
                rows.append((float(m.group(1)), int(m.group(2)), float(m.group(3)),
                             float(m.group(4))))
    return rows


def good_size(n):
    """Smallest even 2^a 3^b 5^c 7^d >= n (and >= 16)."""
    n = max(int(n), 16)
    while True:
        m = n
        if m % 2 == 0:
            for p in (2, 3, 5, 7):
                while m % p == 0:
                    m //= p
            if m == 1:
                return n
        n += 1


def w_range(w, do_wstacking):
    """The w range a plan spans: of |w| with w-stacking (items with w < 0
    are mirrored, :meth:`Plan.coords_lambda`), of w otherwise."""
    a = numpy.abs(w) if do_wstacking else numpy.asarray(w)
    return float(a.min()), float(a.max())


def choose_kernel(epsilon, do_wstacking, sigma=2.0, fp32=False):
    ndim = 3 if do_wstacking else 2
    if fp32 and epsilon < 1e-6:
        raise ValueError("epsilon below 1e-6 needs the FP64 form")
    for s, w, beta, err in es_table():
        if abs(s - sigma) < 1e-9 and ndim * err <= epsilon:
            return w, beta
    raise ValueError("epsilon %g not reachable with sigma %g" % (epsilon, sigma))


class Plan:
    """Plan geometry; mirrors ``gb_plan_geometry`` in the C-ABI."""

    def __init__(self, npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking,
                 w_lo=0.0, w_hi=0.0, sigma=2.0, fp32=False, support=0):
        self.nx, self.ny = npix_x, npix_y
        self.dx, self.dy = pixsize_x, pixsize_y
        self.do_w = bool(do_wstacking)
        if support:
            self.W = support
            self.beta = [b for s, w, b, e in es_table() if abs(s - sigma) < 1e-9 and w == support][0]
        else:
            self.W, self.beta = choose_kernel(epsilon, do_wstacking, sigma, fp32)
        self.sigma = sigma
        self.ngx = good_size(max(math.ceil(sigma * npix_x), 2 * self.W))
        self.ngy = good_size(max(math.ceil(sigma * npix_y), 2 * self.W))
        xm = 0.5 * npix_x * pixsize_x
        ym = 0.5 * npix_y * pixsize_y
        r2 = xm * xm + ym * ym
        if r2 >= 1.0:
            raise ValueError("field of view reaches the horizon")
        if self.do_w:
            tmin = -r2 / (1.0 + math.sqrt(1.0 - r2))
            tmax = 0.0
            self.tc = 0.5 * (tmin + tmax)
            half = 0.5 * (tmax - tmin)
            self.dw = 1.0 / (2.0 * sigma * half)
            self.w_lo = w_lo
            self.nplanes = int(math.ceil((w_hi - w_lo) / self.dw)) + self.W
        else:
            self.tc, self.dw, self.w_lo, self.nplanes = 0.0, 1.0, 0.0, 1

    # -- kernel and correction ------------------------------------------
    def phi(self, x):
        """ES kernel at x in [-1, 1] (support-normalised)."""
        x = numpy.asarray(x, dtype=numpy.float64)
        out = numpy.zeros_like(x)
        inside = numpy.abs(x) < 1.0
        out[inside] = numpy.exp(self.beta * (numpy.sqrt(1.0 - x[inside] ** 2) - 1.0))
        return out

    def phihat(self, nu, nquad=None):
        """Fourier transform of the kernel at nu cycles per cell (Gauss-Legendre)."""
        W = self.W
        nq = nquad or (2 * W + 16)
        xg, wg = numpy.polynomial.legendre.leggauss(2 * nq)
        xg, wg = xg[nq:], wg[nq:]          # half interval, kernel is even
        xs = xg * W / 2.0
        vals = wg * (W / 2.0) * self.phi(xg)
        nu = numpy.asarray(nu, dtype=numpy.float64)
        return 2.0 * numpy.cos(2 * numpy.pi * numpy.multiply.outer(nu, xs)) @ vals

    def pixel_t(self):
        x = (numpy.arange(self.nx) - self.nx // 2) * self.dx
        y = (numpy.arange(self.ny) - self.ny // 2) * self.dy
        xx, yy = numpy.meshgrid(x, y, indexing="ij")
        r2 = xx * xx + yy * yy
        return -r2 / (1.0 + numpy.sqrt(1.0 - r2))

    def correction(self):
        """[nx, ny] factor applied to the plane sum (includes 1/n)."""
        cx = self.phihat((numpy.arange(self.nx) - self.nx // 2) / self.ngx)
        cy = self.phihat((numpy.arange(self.ny) - self.ny // 2) / self.ngy)
        corr = 1.0 / numpy.outer(cx, cy)
        if self.do_w:
            t = self.pixel_t()
            corr = corr / (self.phihat(self.dw * (t - self.tc)) * (1.0 + t))
        return corr

    # -- per-visibility coordinates -------------------------------------
    def coords(self, uvw, freq):
        """Per (row, chan) item: p0, q0 (wrapped), k0, du, dv, dwf, phase,
        flip (see :meth:`coords_lambda`)."""
        s = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
        return self.coords_lambda(uvw[:, 0:1] * s, uvw[:, 1:2] * s, uvw[:, 2:3] * s)

    def coords_lambda(self, u, v, w):
        """Per item with u, v, w in wavelengths: p0, q0 (wrapped), k0, du, dv,
        dwf, phase and flip.  With w-stacking, items with w < 0 are mirrored
        to (-u, -v, -w) (flip True): every image is real, so such an item
        grids conj(value) and predicts the conjugate (Hermitian symmetry),
        and the w range spans |w| only (half the w-planes of a range
        symmetric about zero)."""
        W = self.W
        if self.do_w:
            flip = w < 0.0
            u, v, w = (numpy.where(flip, -x, x) for x in (u, v, w))
        else:
            flip = numpy.zeros(numpy.broadcast(u, v, w).shape, dtype=bool)
        fu = u * self.dx
        fu = fu - numpy.floor(fu)
        U = fu * self.ngx
        p0 = numpy.ceil(U - 0.5 * W)
        du = U - p0
        fv = v * self.dy
        fv = fv - numpy.floor(fv)
        V = fv * self.ngy
        q0 = numpy.ceil(V - 0.5 * W)
        dv = V - q0
        p0 = numpy.mod(p0.astype(numpy.int64), self.ngx)
        q0 = numpy.mod(q0.astype(numpy.int64), self.ngy)
        if self.do_w:
            a = (w - self.w_lo) / self.dw
            k0 = numpy.ceil(a)
            dwf = a - k0 + 0.5 * W
            k0 = numpy.clip(k0.astype(numpy.int64), 0, self.nplanes - W)
            phase = numpy.exp(-2j * numpy.pi * w * self.tc)
        else:
            k0 = numpy.zeros(u.shape, dtype=numpy.int64)
            dwf = numpy.zeros(u.shape)
            phase = numpy.ones(u.shape, dtype=numpy.complex128)
        return p0, q0, k0, du, dv, dwf, phase, flip

    def weights(self, du, dv, dwf):
        """Kernel values [n, W] for u, v and (if w-stacking) w."""
        W = self.W
        a = numpy.arange(W)
        scale = 2.0 / W
        ku = self.phi((a[None, :] - du[:, None]) * scale)
        kv = self.phi((a[None, :] - dv[:, None]) * scale)
        kw = self.phi((a[None, :] - dwf[:, None]) * scale) if self.do_w else numpy.ones((du.size, 1))
        return ku, kv, kw

    def w_plane(self, k):
        return self.w_lo + (k - 0.5 * self.W) * self.dw


def ms2dirty(uvw, freq, ms, wgt, npix_x, npix_y, pixsize_x, pixsize_y, epsilon,
             do_wstacking, sigma=2.0, support=0):
    """Dirty image [npix_x, npix_y] by w-stacking gridding (FP64)."""
    s = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
    w_all = uvw[:, 2:3] * s
    plan = Plan(npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking,
                *w_range(w_all, do_wstacking), sigma, support=support)
    p0, q0, k0, du, dv, dwf, phase, flip = (x.ravel() for x in plan.coords(uvw, freq))
    c = numpy.asarray(ms, dtype=numpy.complex128).ravel()
    if wgt is not None:
        c = c * numpy.asarray(wgt, dtype=numpy.float64).ravel()
    c = numpy.where(flip, numpy.conj(c), c) * phase
    ku, kv, kw = plan.weights(du, dv, dwf)
    W = plan.W
    acc = numpy.zeros((npix_x, npix_y))
    t = plan.pixel_t() if plan.do_w else None
    ox, oy = (plan.ngx - npix_x) // 2, (plan.ngy - npix_y) // 2
    # sign of the checkerboard for every grid cell
    for k in range(plan.nplanes):
        aw = k - k0
        sel = (aw >= 0) & (aw < (W if plan.do_w else 1))
        if not numpy.any(sel):
            continue
        grid = numpy.zeros((plan.ngy, plan.ngx), dtype=numpy.complex128)
        cs = c[sel] * kw[sel, aw[sel]]
        for a in range(W):
            pp = (p0[sel] + a) % plan.ngx
            for b in range(W):
                qq = (q0[sel] + b) % plan.ngy
                sign = 1.0 - 2.0 * ((pp + qq) & 1)
                numpy.add.at(grid, (qq, pp), cs * ku[sel, a] * kv[sel, b] * sign)
        img = numpy.fft.ifft2(grid) * grid.size      # unnormalised e^{+2 pi i}
        block = img[oy:oy + npix_y, ox:ox + npix_x].T  # -> [x, y]
        if plan.do_w:
            block = block * numpy.exp(-2j * numpy.pi * plan.w_plane(k) * (t - plan.tc))
        acc += block.real
    return acc * plan.correction()


def dirty2ms(uvw, freq, dirty, wgt, pixsize_x, pixsize_y, epsilon, do_wstacking,
             sigma=2.0, support=0):
    """Visibilities [nrow, nchan] by w-stacking degridding (FP64)."""
    npix_x, npix_y = dirty.shape
    s = numpy.asarray(freq, dtype=numpy.float64) / SPEED_OF_LIGHT
    w_all = uvw[:, 2:3] * s
    plan = Plan(npix_x, npix_y, pixsize_x, pixsize_y, epsilon, do_wstacking,
                *w_range(w_all, do_wstacking), sigma, support=support)
    p0, q0, k0, du, dv, dwf, phase, flip = (x.ravel() for x in plan.coords(uvw, freq))
    ku, kv, kw = plan.weights(du, dv, dwf)
    W = plan.W
    out = numpy.zeros(p0.size, dtype=numpy.complex128)
    base = numpy.asarray(dirty, dtype=numpy.float64) * plan.correction()
    t = plan.pixel_t() if plan.do_w else None
    ox, oy = (plan.ngx - npix_x) // 2, (plan.ngy - npix_y) // 2
    for k in range(plan.nplanes):
        aw = k - k0
        sel = (aw >= 0) & (aw < (W if plan.do_w else 1))
        if not numpy.any(sel):
            continue
        img = base.astype(numpy.complex128)
        if plan.do_w:
            img = img * numpy.exp(2j * numpy.pi * plan.w_plane(k) * (t - plan.tc))
        z = numpy.zeros((plan.ngy, plan.ngx), dtype=numpy.complex128)
        z[oy:oy + npix_y, ox:ox + npix_x] = img.T
        grid = numpy.fft.fft2(z)
        acc = numpy.zeros(int(sel.sum()), dtype=numpy.complex128)
        for a in range(W):
            pp = (p0[sel] + a) % plan.ngx
            for b in range(W):
                qq = (q0[sel] + b) % plan.ngy
                sign = 1.0 - 2.0 * ((pp + qq) & 1)
                acc += grid[qq, pp] * ku[sel, a] * kv[sel, b] * sign
        out[sel] += acc * kw[sel, aw[sel]]
    out = out * numpy.conj(phase)
    out = numpy.where(flip, numpy.conj(out), out)
    out = out.reshape(uvw.shape[0], len(freq))
    if wgt is not None:
        out = out * wgt
    return out
