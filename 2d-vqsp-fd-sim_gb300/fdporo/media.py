"""Synthetic poroelastic media in the reference's .MO/.JMH form.

The reference reads a per-cell material index JM (.JMH) and a table of 24
coefficients per material (.MO) written by a model-preparation program that
is not part of the repository.  This module derives those coefficients from
Biot's physical parameters, with the meaning the reference's kernels give
them:

* stress (stress_nn.F90:53-55): SIG_XX_1 = SIG_ZZ_2 = lambda_c + 2 mu,
  SIG_XX_2 = SIG_ZZ_1 = lambda_c, SIG_XX_3 = SIG_ZZ_3 = alpha M,
  PRES_1 = PRES_2 = -alpha M, PRES_3 = -M;
* velocity (inh_qx_int.F90:44-52, inh_v_uv_int.F90:45-54), with
  rho = (1-phi) rho_s + phi rho_f, m = T rho_f / phi, D = rho m - rho_f**2,
  b = eta / kappa: REL1_U = m/D, REL2_U = rho_f b/D, REL3_U = rho_f/D,
  REL1_Q = rho_f/D, REL2_Q = rho/D, REL3_Q = rho b/D (unscaled; the
  reference multiplies by DT and divides by H after reading,
  read_model_par.F90:63-74);
* free-surface row (read_model_par.F90:78-87, the commented derivation):
  AUXIL_W = (lambda_c - (alpha M)**2/M) / (lambda_c + 2 mu - (alpha M)**2/M),
  AUXIL_QZ = 2 mu (alpha M / M) / (lambda_c + 2 mu - (alpha M)**2/M).

Gassmann/Biot moduli: alpha = 1 - K_frame/K_s,
M = 1 / ((alpha - phi)/K_s + phi/K_f), lambda_c = K_frame - 2 mu/3 + alpha**2 M.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

# column order of a .MO record (read_model_par.F90:52-60)
MO_COLUMNS = ["MU", "SIG_XX_1", "SIG_XX_2", "SIG_XX_3", "SIG_ZZ_1", "SIG_ZZ_2", "SIG_ZZ_3",
              "PRES_1", "PRES_2", "PRES_3", "REL1_U", "REL1_W", "REL2_U", "REL2_W", "REL3_U", "REL3_W",
              "REL1_QX", "REL1_QZ", "REL2_QX", "REL2_QZ", "REL3_QX", "REL3_QZ", "AUXIL_W", "AUXIL_QZ"]
COL = {n: i for i, n in enumerate(MO_COLUMNS)}


@dataclass(frozen=True)
class Rock:
    """Physical parameters of a Biot medium (SI units)."""
    rho_s: float = 2650.0
    rho_f: float = 1000.0
    phi: float = 0.2
    k_s: float = 37e9
    k_f: float = 2.25e9
    k_frame: float = 10e9
    mu: float = 9e9
    kappa: float = 1e-12
    eta: float = 1e-3
    tortuosity: float = 2.0


# brine-saturated sandstone of the small homogeneous case, and the stiffer
# tight layer of the layered case
SANDSTONE = Rock()
TIGHT_LAYER = replace(SANDSTONE, k_frame=20e9, mu=15e9, phi=0.1, kappa=1e-14)


def biot_table(rho_s, rho_f, phi, k_s, k_f, k_frame, mu, kappa, eta, tortuosity) -> np.ndarray:
    """Unscaled .MO coefficients, shape (..., 24), float64."""
    rho_s, rho_f, phi, k_s, k_f, k_frame, mu, kappa, eta, tortuosity = np.broadcast_arrays(
        *[np.asarray(v, dtype=np.float64) for v in (rho_s, rho_f, phi, k_s, k_f, k_frame, mu, kappa, eta,
                                                     tortuosity)])
    alpha = 1.0 - k_frame / k_s
    M = 1.0 / ((alpha - phi) / k_s + phi / k_f)
    lamc = k_frame - 2.0 * mu / 3.0 + alpha * alpha * M
    l2mc = lamc + 2.0 * mu
    am = alpha * M
    rho = (1.0 - phi) * rho_s + phi * rho_f
    m = tortuosity * rho_f / phi
    delta = rho * m - rho_f * rho_f
    b = eta / kappa
    dry = l2mc - am * am / np.where(M == 0, 1.0, M)
    auxw = np.where(M == 0, lamc / l2mc, (lamc - am * am / np.where(M == 0, 1.0, M)) / dry)
    auxqz = np.where(M == 0, 0.0, (am / np.where(M == 0, 1.0, M)) * 2.0 * mu / dry)
    col = {"MU": mu, "SIG_XX_1": l2mc, "SIG_XX_2": lamc, "SIG_XX_3": am, "SIG_ZZ_1": lamc, "SIG_ZZ_2": l2mc,
           "SIG_ZZ_3": am, "PRES_1": -am, "PRES_2": -am, "PRES_3": -M, "AUXIL_W": auxw, "AUXIL_QZ": auxqz}
    for s in ("U", "W"):
        col["REL1_" + s] = m / delta
        col["REL2_" + s] = rho_f * b / delta
        col["REL3_" + s] = rho_f / delta
    for s in ("QX", "QZ"):
        col["REL1_" + s] = rho_f / delta
        col["REL2_" + s] = rho / delta
        col["REL3_" + s] = rho * b / delta
    # one pass into the interleaved (..., 24) layout
    return np.stack([np.asarray(col[n], dtype=np.float64) for n in MO_COLUMNS], axis=-1)


def rock_table(rock: Rock) -> np.ndarray:
    return biot_table(rock.rho_s, rock.rho_f, rock.phi, rock.k_s, rock.k_f, rock.k_frame, rock.mu,
                      rock.kappa, rock.eta, rock.tortuosity)


def gaussian_random_field(shape: tuple[int, int], corr_len_cells: float, seed: int) -> np.ndarray:
    """Unit-variance stationary Gaussian field with a Gaussian correlation of
    length ``corr_len_cells``, made by filtering white noise in the Fourier
    domain (numpy ``default_rng(seed)``)."""
    rng = np.random.default_rng(seed)
    nz, nx = shape
    noise = rng.standard_normal((nz, nx))
    kz = np.fft.fftfreq(nz)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    # spectrum of exp(-r^2/l^2) is proportional to exp(-(pi l k)^2)
    amp = np.exp(-0.5 * (np.pi * corr_len_cells) ** 2 * (kz * kz + kx * kx))
    f = np.fft.irfft2(np.fft.rfft2(noise) * amp, s=(nz, nx))
    f -= f.mean()
    sd = f.std()
    return f / sd if sd > 0 else f


@dataclass
class Medium:
    """A medium as the reference's input files hold it: the physical JM rows
    (as read from .JMH, rows 2..MZ under stress imaging) and the unscaled
    .MO table (jmnum, 24)."""
    jm_rows: np.ndarray   # (n_rows, mx) int32, values 1..jmnum
    table: np.ndarray     # (jmnum, 24) float64

    @property
    def jmnum(self) -> int:
        return int(self.table.shape[0])


def homogeneous(mx: int, n_rows: int, rock: Rock = SANDSTONE) -> Medium:
    return Medium(np.ones((n_rows, mx), dtype=np.int32), rock_table(rock)[None, :])


def layered_grf(mx: int, n_rows: int, h: float, seed: int, layer_depth: float = 1024.0,
                upper: Rock = SANDSTONE, lower: Rock = TIGHT_LAYER, std: float = 0.1,
                corr_len: float = 20.0) -> Medium:
    """Two layers (``upper`` above depth ``layer_depth``) with K_frame, mu and
    phi each multiplied by (1 + std*g), g a unit-variance Gaussian random
    field of correlation length ``corr_len`` metres; one material per cell
    (JMNUM = cells)."""
    depth = np.arange(n_rows, dtype=np.float64)[:, None] * h
    low = depth >= layer_depth
    g = gaussian_random_field((n_rows, mx), corr_len / h, seed)
    t = np.empty((n_rows, mx, 24), dtype=np.float64)
    # blocks of rows, so that the element-wise temporaries stay small on
    # large grids (the values do not depend on the blocking)
    step = max(1, (1 << 22) // max(mx, 1))
    for r0 in range(0, n_rows, step):
        r1 = min(n_rows, r0 + step)
        fac = 1.0 + std * g[r0:r1]

        def pick(name):
            a, b = getattr(upper, name), getattr(lower, name)
            return np.where(low[r0:r1], b, a) * np.ones((r1 - r0, mx))

        t[r0:r1] = biot_table(pick("rho_s"), pick("rho_f"), pick("phi") * fac, pick("k_s"), pick("k_f"),
                              pick("k_frame") * fac, pick("mu") * fac, pick("kappa"), pick("eta"),
                              pick("tortuosity"))
    jm = (np.arange(n_rows * mx, dtype=np.int32) + 1).reshape(n_rows, mx)
    return Medium(jm, t.reshape(-1, 24))
