"""ORACLE (test infrastructure only): restatement of FDFK2D's FK background wavefield.

`comput_background_wavefield_` (call site src/FDFK2D.f90:432-434) ships closed in
lib_gnu/libFK3D.so.  Its algorithm, recovered by running it as a black box
(oracle/refharness.py observes the FFTs and LU solves it makes through shims
written here), is restated below in NumPy (FP64, complex):

* source time function: w(t_n) = ds * Ricker(f0; t_n - 1.25/f0) * exp(-alpha t_n),
  n = 0..nt, zero after; alpha = 10 / (nt dt) (complex-frequency damping);
* N = smallest power of two >= 2 (nt + 1); W = forward DFT of w (sign -1);
  frequencies above 10 f0 are set to zero;
* per strip point (x, z) and component: X(omega_k) = W_k * U(x, z; omega_k - i alpha),
  U = plane-wave response of the 1-D layered model with a free surface to a
  unit incident wave from the bottom half-space, evaluated at complex
  frequency; horizontal phase p (cos(baz_j) (x - x_c) - x_c' |cos(baz_mean)|)
  with x_c the profile centre and x_c' = (nx - 1) dx / 2 (for back-azimuth 0
  the phase is zero at column nx and the wave travels towards -x); vertical
  phase zero at row nz;
* strip value s(t_n) = Re(IDFT(X))_n * exp(alpha t_n) / N (IDFT sign +1), n = 0..nt;
* model: left strips use the left model, right strips the right model; bottom
  strips use the model of the side the wave arrives from, except the nbd
  columns below the other side strip, which use that side's model.

The plane-wave response is solved with a global matrix per frequency
(continuity of displacement and traction at every interface, zero traction at
the surface); the reference solves the same boundary-value problem with 4x4
propagator matrices, so the two agree to rounding while the problem is well
conditioned.  Beyond the P critical slowness of the half-space (S incidence with
p well above 1/vp there) the reference's output grows without bound (1e8 to 1e33
in probes) and is not reproduced; that regime is outside what this oracle pins.
"""
from __future__ import annotations

import numpy as np

# Incident amplitude in this module's polarisation convention (the reference's sign).
INC_AMP = {"P": -1.0, "S": -1.0}

STRIPS = ("uxl_reg", "uzl_reg", "uxr_reg", "uzr_reg", "uxb_reg", "uzb_reg",
          "uxl_pml", "uzl_pml", "uxr_pml", "uzr_pml", "uxb_pml", "uzb_pml")


def nfft(nt: int) -> int:
    n = 1
    while n < 2 * (nt + 1):
        n *= 2
    return n


def source_spectrum(nt, dt, f0, ds):
    """Forward DFT of the damped, delayed Ricker source, its length N and the damping alpha."""
    N = nfft(nt)
    alpha = 10.0 / (nt * dt)
    t = np.arange(N) * dt
    f0 = float(np.float32(f0))
    a = (np.pi * f0 * (t - 1.25 / f0)) ** 2
    w = float(np.float32(ds)) * (1.0 - 2.0 * a) * np.exp(-a) * np.exp(-alpha * t)   # ds is single precision
    w[nt + 1:] = 0.0
    return np.fft.fft(w), N, alpha


def strip_coords(nx, nz, nbd, name):
    """Fortran (iz, ix) index vectors of a background strip (src/FDFK2D.f90:328-355)."""
    side, kind = name[2], name[4:]
    if kind == "reg":
        if side == "l":
            return np.arange(1, nz - nbd + 1), np.arange(1, nbd + 1)
        if side == "r":
            return np.arange(1, nz - nbd + 1), np.arange(nx - nbd + 1, nx + 1)
        return np.arange(nz - nbd + 1, nz + 1), np.arange(1, nx + 1)
    if side == "l":
        return np.arange(1, nz + 1), np.arange(1 - nbd, 1)
    if side == "r":
        return np.arange(1, nz + 1), np.arange(nx + 1, nx + nbd + 1)
    return np.arange(nz + 1, nz + nbd + 1), np.arange(1 - nbd, nx + nbd + 1)


def layered_response(model, p, wc, z, incident="P", z_ref=0.0):
    """Radial and vertical displacement U_R, U_Z (len(wc) x len(z)) of a unit plane wave.

    model: (4, L) = z_top, vp, vs, rho per layer (layer L-1 is the half-space).
    The incident wave (P or SV) travels upward in the half-space with radial
    slowness p; its amplitude is 1 with phase zero at depth z_ref.  z is down;
    fields vary as exp(i (w t + w p r +- w q z)) with r the horizontal coordinate
    along the back-azimuth (the wave moves towards -r).
    """
    zt = np.asarray(model[0], np.float64)
    vp = np.asarray(model[1], np.float64)
    vs = np.asarray(model[2], np.float64)
    rho = np.asarray(model[3], np.float64)
    L = len(zt)
    sx = -float(p)
    # vertical slownesses, principal square root (an evanescent wave labelled "down"
    # grows with depth, as in the reference)
    eta = np.sqrt(1.0 / vp ** 2 - sx * sx + 0j)
    nu = np.sqrt(1.0 / vs ** 2 - sx * sx + 0j)
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2.0 * mu

    def wave(j, k):
        """vertical slowness and [ux, uz, sxz/(-iw), szz/(-iw)] per unit amplitude."""
        a, b = vp[j], vs[j]
        if k == 0:
            sz, pol = eta[j], (sx * a, eta[j] * a)          # down P
        elif k == 1:
            sz, pol = nu[j], (nu[j] * b, -sx * b)           # down SV
        elif k == 2:
            sz, pol = -eta[j], (sx * a, -eta[j] * a)        # up P
        else:
            sz, pol = -nu[j], (nu[j] * b, sx * b)           # up SV
        sxz = mu[j] * (sz * pol[0] + sx * pol[1])
        szz = lam[j] * sx * pol[0] + (lam[j] + 2.0 * mu[j]) * sz * pol[1]
        return sz, np.array([pol[0], pol[1], sxz, szz], complex)

    waves = [[wave(j, k) for k in range(4)] for j in range(L)]
    inc = 2 if incident == "P" else 3
    n = 4 * (L - 1) + 2

    def col(j, k):
        if j < L - 1:
            return 4 * j + k
        return 4 * (L - 1) + k if k < 2 else None

    nw = len(wc)
    amps = np.zeros((nw, L, 4), complex)
    for iw, w in enumerate(wc):
        A = np.zeros((n, n), complex)
        rhs = np.zeros(n, complex)
        r = 0
        for comp in (2, 3):                                  # free surface, z = 0
            for k in range(4):
                sz, v = waves[0][k]
                term = v[comp] * np.exp(-1j * w * sz * (0.0 - zt[0]))
                c = col(0, k)
                if c is not None:
                    A[r, c] += term
                elif k == inc:
                    rhs[r] -= term
            r += 1
        for j in range(L - 1):                               # interface at zt[j+1]
            zi = zt[j + 1]
            for comp in range(4):
                for k in range(4):
                    sz, v = waves[j][k]
                    A[r, col(j, k)] += v[comp] * np.exp(-1j * w * sz * (zi - zt[j]))
                    sz2, v2 = waves[j + 1][k]
                    term = v2[comp]                          # phase 1 at the top of layer j+1
                    c2 = col(j + 1, k)
                    if c2 is not None:
                        A[r, c2] -= term
                    elif k == inc:
                        rhs[r] += term
                r += 1
        x = np.linalg.solve(A, rhs * INC_AMP[incident])
        for j in range(L):
            for k in range(4):
                c = col(j, k)
                if c is not None:
                    amps[iw, j, k] = x[c]
        amps[iw, L - 1, inc] = INC_AMP[incident]
    # incident phase zero at z_ref: scale everything by exp(-i w sz_inc (zt[L-1] - z_ref))
    sz_inc = waves[L - 1][inc][0]
    amps *= np.exp(-1j * wc * sz_inc * (zt[L - 1] - z_ref))[:, None, None]
    z = np.asarray(z, np.float64)
    lay = np.clip(np.searchsorted(zt, z, side="right") - 1, 0, L - 1)
    UR = np.zeros((nw, len(z)), complex)
    UZ = np.zeros((nw, len(z)), complex)
    for iz, (zz, j) in enumerate(zip(z, lay)):
        for k in range(4):
            sz, v = waves[j][k]
            e = amps[:, j, k] * np.exp(-1j * wc * sz * (zz - zt[j]))
            UR[:, iz] += e * v[0]
            UZ[:, iz] += e * v[1]
    return UR, UZ


def background(p, bazs, fk_left, fk_right, x0=0.0, z0=0.0, dtype=np.float32):
    """Restated comput_background_wavefield: dict of the 12 strips (n1, n2, nt+1), float32 as the
    reference stores them (dtype=np.float64 keeps the FP64 values, for the FP64 oracle).

    p: nx, nz, npml, nbd, nt, dt, dx, dz, f0, ds, rayp (s/m), src_type (True = P).
    bazs: back-azimuths (rad) of the nx + 2 npml columns, profile frame.
    Model per column: the left strips use fk_left, the right strips fk_right;
    the bottom strips use the model of the side the wave comes from, except the
    nbd columns under the far side strip: for cos(baz_mean) >= 0 (wave moving
    towards -x) fk_left for ix <= nbd and fk_right beyond, otherwise fk_right
    for ix > nx - nbd and fk_left before.
    """
    nx, nz, npml, nbd, nt, dt = p["nx"], p["nz"], p["npml"], p["nbd"], p["nt"], p["dt"]
    dx, dz = p["dx"], p["dz"]
    W, N, alpha = source_spectrum(nt, dt, p["f0"], p["ds"])
    nh = N // 2
    # frequencies above 10 f0 are dropped
    kmax = min(nh - 1, int(np.floor(10.0 * float(np.float32(p["f0"])) * N * dt)))
    w = 2.0 * np.pi * np.arange(nh + 1) / (N * dt)
    wc = w - 1j * alpha
    inc = "P" if p["src_type"] else "S"
    ray = float(p["rayp"])
    # Horizontal phase: each column is projected on its own back-azimuth about the
    # profile centre x_c; the reference is the end the wave reaches first, projected
    # on the mean back-azimuth (the mean divides by nx + 2 npml + 1, as the
    # reference's own check at src/FDFK2D.f90:388 does).
    x_c = x0 + 0.5 * (nx - 1) * dx
    half = 0.5 * (nx - 1) * dx
    cbar = np.cos(np.sum(np.asarray(bazs, np.float64)) / (nx + 2 * npml + 1))
    r_ref = half * abs(cbar)
    z_ref = z0 + (nz - 1) * dz
    tn = np.arange(nt + 1) * dt
    out = {}
    cache = {}
    for name in STRIPS:
        iz, ix = strip_coords(nx, nz, nbd, name)
        side = name[2]
        arr = np.zeros((len(iz), len(ix), nt + 1), dtype, order="F")
        for jj, cx in enumerate(ix):
            if side == "b":
                left = cx <= nbd if cbar >= 0.0 else cx <= nx - nbd
            else:
                left = side == "l"
            model = fk_left if left else fk_right
            key = (id(model), tuple(iz))
            if key not in cache:
                cache[key] = layered_response(model, ray, wc, z0 + (iz - 1) * dz, inc, z_ref)
            UR, UZ = cache[key]
            phi = float(bazs[cx - 1 + npml])
            x = x0 + (cx - 1) * dx
            ph = np.exp(1j * wc * ray * (np.cos(phi) * (x - x_c) - r_ref))
            U = UR * np.cos(phi) if name[1] == "x" else UZ
            X = np.zeros((N, len(iz)), complex)
            X[:kmax + 1] = W[:kmax + 1, None] * U[:kmax + 1] * ph[:kmax + 1, None]
            X[N - kmax:] = np.conj(X[1:kmax + 1][::-1])
            xt = np.fft.ifft(X, axis=0).real * N
            arr[:, jj, :] = (xt[:nt + 1].T * np.exp(alpha * tn) / N).astype(dtype)
        out[name] = arr
    return out


def background_device(p, bazs, fk_left, fk_right, x0=0.0, z0=0.0, device="cuda", chunk_bytes=1 << 30):
    """:func:`background` in FP64 with the per-column inverse transforms batched on a torch device.

    Same mathematics as :func:`background` (same spectrum, response, phase, fold and scaling): the
    layered response is evaluated only at the kept frequencies (k <= 10 f0 N dt; the others are
    zero in both), and the inverse transform of the Hermitian spectrum is a real inverse FFT.
    Returns dict name -> float64 tensor of shape (nt+1, n2, n1), C-contiguous: the bytes of the
    reference's Fortran strip (n1, n2, nt+1).  Used for the FP64 oracle at full workload sizes.
    """
    import torch
    nx, nz, npml, nbd, nt, dt = p["nx"], p["nz"], p["npml"], p["nbd"], p["nt"], p["dt"]
    dx, dz = p["dx"], p["dz"]
    W, N, alpha = source_spectrum(nt, dt, p["f0"], p["ds"])
    nh = N // 2
    kmax = min(nh - 1, int(np.floor(10.0 * float(np.float32(p["f0"])) * N * dt)))
    w = 2.0 * np.pi * np.arange(nh + 1) / (N * dt)
    wc = (w - 1j * alpha)[:kmax + 1]
    inc = "P" if p["src_type"] else "S"
    ray = float(p["rayp"])
    x_c = x0 + 0.5 * (nx - 1) * dx
    half = 0.5 * (nx - 1) * dx
    cbar = np.cos(np.sum(np.asarray(bazs, np.float64)) / (nx + 2 * npml + 1))
    r_ref = half * abs(cbar)
    z_ref = z0 + (nz - 1) * dz
    tn = torch.arange(nt + 1, dtype=torch.float64, device=device) * dt
    damp = torch.exp(alpha * tn)
    Wt = torch.as_tensor(W[:kmax + 1], device=device)
    wct = torch.as_tensor(wc, device=device)
    out = {}
    cache = {}
    for name in STRIPS:
        iz, ix = strip_coords(nx, nz, nbd, name)
        side = name[2]
        res = torch.empty((nt + 1, len(ix), len(iz)), dtype=torch.float64, device=device)
        groups = {}
        for jj, cx in enumerate(ix):
            if side == "b":
                left = cx <= nbd if cbar >= 0.0 else cx <= nx - nbd
            else:
                left = side == "l"
            groups.setdefault(bool(left), []).append(jj)
        for left, cols in groups.items():
            model = fk_left if left else fk_right
            key = (id(model), tuple(iz))
            if key not in cache:
                UR, UZ = layered_response(model, ray, wc, z0 + (iz - 1) * dz, inc, z_ref)
                cache[key] = (torch.as_tensor(UR, device=device), torch.as_tensor(UZ, device=device))
            UR, UZ = cache[key]
            per_col = (nh + 1) * len(iz) * 16 + N * len(iz) * 8
            step = max(1, int(chunk_bytes // per_col))
            for a in range(0, len(cols), step):
                cj = cols[a:a + step]
                cxs = np.asarray([ix[j] for j in cj])
                phi = np.asarray(bazs, np.float64)[cxs - 1 + npml]
                xs = x0 + (cxs - 1) * dx
                arg = torch.as_tensor(ray * (np.cos(phi) * (xs - x_c) - r_ref), device=device)
                ph = torch.exp(1j * wct[:, None] * arg[None, :])                       # (K, C)
                if name[1] == "x":
                    U = UR[:, :, None] * torch.as_tensor(np.cos(phi), device=device)[None, None, :]
                else:
                    U = UZ[:, :, None].expand(-1, -1, len(cj))
                X = torch.zeros((nh + 1, len(iz), len(cj)), dtype=torch.complex128, device=device)
                X[:kmax + 1] = Wt[:, None, None] * U * ph[:, None, :]
                xt = torch.fft.irfft(X, n=N, dim=0) * N                                  # (N, R, C)
                del X
                v = xt[:nt + 1] * damp[:, None, None] / N
                res[:, cj[0]:cj[-1] + 1, :] = v.permute(0, 2, 1)
                del xt, v
        out[name] = res
    return out
