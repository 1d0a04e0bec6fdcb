"""Second, independent CPU oracle: numpy restatement of InstaHeat's mk_rhs.

TEST INFRASTRUCTURE ONLY.  Written directly from nikikilbertus/InstaHeat
src/toolbox.c (mk_rhs 75-88, mk_gradient_squared_and_laplacian 129-149,
mk_ffts_and_filter 160-186, mk_rho_and_p 225-243, update_phi_psi 282-299,
update_h 311-346, mk_gw_sources_tt 363-397, mk_gw_spectrum 435-484,
mk_constraints 524-551, mk_power_spectrum 567-582) and src/setup.c
(mk_k_grid 609-666, mk_filter_mask 710-754), using numpy.fft (pocketfft)
in place of FFTW.  It cross-checks the C oracle on small grids.
"""
from __future__ import annotations

import numpy as np

EPS = np.finfo(np.float64).eps


def kgrid(n, L):
    nx, ny, nz = n
    ux, uy, uz = (2 * np.pi / L[0], 2 * np.pi / L[1], 2 * np.pi / L[2])

    def axis(N, u, half=False):
        idx = np.arange(N // 2 + 1) if half else np.arange(N)
        kf = np.where(idx > N // 2, idx - N, idx).astype(float) * u
        k = np.where(2 * idx == N, 0.0, kf)
        return k, kf

    kx, kxf = axis(nx, ux)
    ky, kyf = axis(ny, uy)
    kz, kzf = axis(nz, uz, half=True)
    sh = (nx, ny, nz // 2 + 1)
    g = {
        "x": np.broadcast_to(kx[:, None, None], sh).copy(),
        "y": np.broadcast_to(ky[None, :, None], sh).copy(),
        "z": np.broadcast_to(kz[None, None, :], sh).copy(),
        "xf": np.broadcast_to(kxf[:, None, None], sh).copy(),
        "yf": np.broadcast_to(kyf[None, :, None], sh).copy(),
        "zf": np.broadcast_to(kzf[None, None, :], sh).copy(),
    }
    g["sq"] = g["xf"] ** 2 + g["yf"] ** 2 + g["zf"] ** 2
    kmax = np.sqrt((ux * (nx // 2)) ** 2 + (uy * (ny // 2)) ** 2 + (uz * (nz // 2)) ** 2)
    return g, kmax


def filter_mask(n, L, g):
    kxm = (n[0] // 2) * 2 * np.pi / L[0]
    kym = (n[1] // 2) * 2 * np.pi / L[1]
    kzm = (n[2] // 2) * 2 * np.pi / L[2]
    frac = np.maximum(np.maximum(np.abs(g["xf"]) / kxm, np.abs(g["yf"]) / kym), np.abs(g["zf"]) / kzm)
    return np.exp(-36.0 * frac ** 36)


class NumpyRHS:
    def __init__(self, n, L, mass=1.0, gw=True, filter=True, bins=None):
        self.n, self.L, self.m = tuple(n), tuple(L), mass
        self.gw, self.filter_enabled = gw, filter
        self.bins = bins if bins is not None else n[0] // 2
        self.N = n[0] * n[1] * n[2]
        self.M = n[0] * n[1] * (n[2] // 2 + 1)
        self.Next = 2 * self.M
        self.Ntot = 4 * self.N + 4 * self.Next + 1
        self.g, self.kmax = kgrid(n, L)
        self.mask = filter_mask(n, L, self.g)

    def fft(self, x):
        return np.fft.rfftn(x.reshape(self.n))

    def ifft(self, c):
        return np.fft.irfftn(c, s=self.n, axes=(0, 1, 2)) * self.N

    def rhs(self, f, filter=0, output=0):
        """Returns (result, filtered f, diag dict)."""
        f = np.array(f, dtype=float, copy=True)
        N, Next, M = self.N, self.Next, self.M
        g = self.g
        phi, dphi, psi, dpsi = (f[i * N:(i + 1) * N] for i in range(4))
        a = f[-1]
        a2 = a * a
        diag = {}
        phic = self.fft(phi)
        psic = None
        if self.filter_enabled:
            if filter:
                psic = self.fft(psi)
                phic = phic * self.mask
                psic = psic * self.mask
                phi[:] = self.ifft(phic / N).ravel()
                psi[:] = self.ifft(psic / N).ravel()
                dphi[:] = self.ifft(self.fft(dphi) * self.mask / N).ravel()
                dpsi[:] = self.ifft(self.fft(dpsi) * self.mask / N).ravel()
        elif output:
            psic = self.fft(psi)
        lap_psi = self.ifft(-psic * g["sq"] / N).ravel() if output else None
        pre = phic / N
        xphi = self.ifft(pre * 1j * g["x"]).ravel()
        yphi = self.ifft(pre * 1j * g["y"]).ravel()
        zphi = self.ifft(pre * 1j * g["z"]).ravel()
        lap = self.ifft(-pre * g["sq"]).ravel()
        grad = xphi ** 2 + yphi ** 2 + zphi ** 2
        V = self.m ** 2 * phi ** 2 / 2
        t1 = (0.5 - psi) * dphi ** 2
        t2 = (0.5 + psi) * grad / a2
        rho = t1 + t2 + V
        p = t1 - t2 / 3.0 - V
        rho_mean, p_mean = rho.mean(), p.mean()
        H = np.sqrt(rho_mean / 3.0)
        res = np.zeros(self.Ntot)
        res[:N] = dphi
        res[N:2 * N] = (1 + 4 * psi) * lap / a2 - (3 * H - 4 * dpsi) * dphi - (1 + 2 * psi) * self.m ** 2 * phi
        res[2 * N:3 * N] = dpsi
        res[3 * N:4 * N] = 0.5 * p + (psi - 0.5) * p_mean - 4 * H * dpsi
        if self.gw:
            h = [f[4 * N + j * Next: 4 * N + (j + 1) * Next].view(np.complex128).reshape(phic.shape) for j in range(4)]
            res[4 * N:4 * N + 2 * Next] = f[4 * N + 2 * Next:4 * N + 4 * Next]
            st = self.tt_sources(xphi, yphi, zphi)
            tm = -(2 * p_mean + g["sq"] / a2)
            dd1 = tm * h[0] - 3 * H * h[2] + 2 * st[0] / a2
            dd2 = tm * h[1] - 3 * H * h[3] + 2 * st[1] / a2
            res[4 * N + 2 * Next:4 * N + 3 * Next] = dd1.ravel().view(np.float64)
            res[4 * N + 3 * Next:4 * N + 4 * Next] = dd2.ravel().view(np.float64)
        res[-1] = a * H
        if output:
            diag["phi_ps"] = self.power_spectrum(phic)
            diag["psi_ps"] = self.power_spectrum(psic)
            diag["rho_ps"] = self.power_spectrum(self.fft(rho))
            t1c = H * psi + dpsi
            ham = lap_psi / a2 - 3 * H * t1c - 0.5 * (rho - rho_mean)
            mom = t1c - 0.5 * dphi.mean() * (phi - phi.mean())
            diag["cstr"] = np.array([np.mean(ham ** 2), np.abs(ham).max(), np.mean(mom ** 2), np.abs(mom).max()])
            if self.gw:
                diag["gw"] = self.gw_spectrum(f, H)
        diag.update(rho_mean=rho_mean, pressure_mean=p_mean, lap=lap, grad=grad, rho=rho, p=p)
        return res, f, diag

    def tt_sources(self, xphi, yphi, zphi):
        d = [xphi, yphi, zphi]
        pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
        s = [self.fft(d[i] * d[j]) for i, j in pairs]
        g = self.g
        kx, ky, kz, ksq = g["xf"], g["yf"], g["zf"], g["sq"].copy()
        ksq.flat[0] = 1.0
        fx, fy, fz = kx / ksq, ky / ksq, kz / ksq
        t1 = kx * fx * s[0] + ky * fy * s[3] + kz * fz * s[5] + 2 * (kx * fy * s[1] + kx * fz * s[2] + ky * fz * s[4])
        t2 = s[0] + s[3] + s[5]
        S1, S2 = t1 + t2, t1 - t2
        k1 = kx * s[0] + ky * s[1] + kz * s[2]
        k2 = kx * s[1] + ky * s[3] + kz * s[4]
        k3 = kx * s[2] + ky * s[4] + kz * s[5]
        bz = np.abs(kz) > EPS
        by = (~bz) & (np.abs(ky) > EPS)
        bo = (~bz) & (~by)
        n0 = np.where(bo, s[3] - 2 * fy * k2 + 0.5 * (fy * ky * S1 + S2),
                      s[0] - 2 * fx * k1 + 0.5 * (fx * kx * S1 + S2))
        n1 = np.where(bz, s[1] - fx * k2 - fy * k1 + 0.5 * fx * ky * S1,
                      np.where(by, s[2] - fx * k3 - fz * k1 + 0.5 * fx * kz * S1,
                               s[4] - fy * k3 - fz * k2 + 0.5 * fy * kz * S1))
        n0.flat[0] = 0.0
        n1.flat[0] = 0.0
        return n0, n1

    def _bin_index(self, k):
        # |k| = k_max stays in the last bin where the offset is lost to
        # rounding (toolbox.c:479 would index one past its array there)
        return np.minimum(np.trunc(self.bins * k / self.kmax - 1.0e-14).astype(int),
                          self.bins - 1)

    def power_spectrum(self, c):
        p2 = (np.abs(c) ** 2).ravel().copy()
        p2[np.abs(self.g["z"]).ravel() > EPS] *= 2.0
        idx = self._bin_index(np.sqrt(self.g["sq"].ravel()))
        out = np.zeros(self.bins)
        np.add.at(out, idx[1:], p2[1:] / self.N)
        return out

    def gw_spectrum(self, f, H):
        N, Next = self.N, self.Next
        d1 = f[4 * N + 2 * Next:4 * N + 3 * Next].view(np.complex128)
        d2 = f[4 * N + 3 * Next:4 * N + 4 * Next].view(np.complex128)
        g = self.g
        kx, ky, kz = g["xf"].ravel(), g["yf"].ravel(), g["zf"].ravel()
        kx2, ky2, kz2 = kx ** 2, ky ** 2, kz ** 2
        k2 = g["sq"].ravel()
        k = np.sqrt(k2)
        a1 = np.abs(d1) ** 2
        a2 = np.abs(d2) ** 2
        x12 = (d1.real * d2.real + d1.imag * d2.imag)
        with np.errstate(divide="ignore", invalid="ignore"):
            pz = 2 * k2 / (kz2 * (ky2 + kz2)) * ((kx2 + kz2) * a1 + 2 * kx * ky * x12 + (ky2 + kz2) * a2)
            py = 2 * (kx2 + ky2) / (ky2 * ky2) * ((kx2 + ky2) * a1 + ky2 * a2)
        po = 2 * (a1 + a2)
        bz = np.abs(kz) > EPS
        by = (~bz) & (np.abs(ky) > EPS)
        pw = np.where(bz, pz, np.where(by, py, po))
        pw = np.where(np.abs(g["z"].ravel()) > EPS, 2 * pw, pw)
        fac = np.pi * 0.01 ** (1 / 3) / (3 * H * H * self.L[0] * self.L[1] * self.L[2])
        idx = self._bin_index(k)
        out = np.zeros(self.bins)
        np.add.at(out, idx[1:], (fac * k2 * k * pw)[1:])
        return out / N
