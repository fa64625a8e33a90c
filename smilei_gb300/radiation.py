"""Monte-Carlo radiation reaction on the GPU: tables, the Monte-Carlo pass and the MLP surrogate.

``RadiationTables`` mirrors the reference's RadiationTables (tables in its
conventions, src/Radiation/RadiationTables.h); ``monte_carlo`` runs
RadiationMonteCarlo::operator() over a species' particles;
``PhotonChiMLP`` is the learned inverse CDF (hand-written CUDA training and
inference in csrc/radiation.cu) with the table as fallback and as its check.
All arrays are torch CUDA tensors (float64).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr

# Physical constants (SI) used to derive the normalised factors exactly as
# RadiationTables::initialization and Radiation's constructor do
# (RadiationTables.cpp:92-103, Radiation.cpp:29-33).
RED_PLANCK = 1.054571817e-34
ELECTRON_MASS = 9.1093837015e-31
C_VACUUM = 299792458.0
FINE_STRUCTURE = 7.2973525693e-3


def normalised_factors(reference_angular_frequency_SI: float):
    """(factor_dNph_dt, factor_classical_radiated_power, inv_norm_E_Schwinger) for omega_r."""
    lam = RED_PLANCK * reference_angular_frequency_SI / (ELECTRON_MASS * C_VACUUM ** 2)
    f_dn = np.sqrt(3.0) * FINE_STRUCTURE / (2.0 * np.pi * lam)
    f_cl = 2.0 * FINE_STRUCTURE / (3.0 * lam)
    inv_es = lam  # 1 / (m c^2 / (hbar omega_r))
    return f_dn, f_cl, inv_es


class RadiationTables:
    def __init__(self, integfochi, integ_min, integ_max, xi, xi_min, xi_max, axis1_min, factor_dNph_dt,
                 factor_classical, inv_norm_E_schwinger, min_chi_continuous=1e-3, min_chi_discontinuous=1e-2):
        integ = np.ascontiguousarray(integfochi, dtype=np.float64)
        xi = np.ascontiguousarray(xi, dtype=np.float64)
        ax = np.ascontiguousarray(axis1_min, dtype=np.float64)
        fac = np.array([factor_dNph_dt, factor_classical, inv_norm_E_schwinger, min_chi_continuous,
                        min_chi_discontinuous], dtype=np.float64)
        h = ctypes.c_void_p()
        check(_lib.lib().sg_rad_tables_create(integ.ctypes.data, len(integ), float(integ_min), float(integ_max),
                                              xi.ctypes.data, xi.shape[0], xi.shape[1], float(xi_min),
                                              float(xi_max), ax.ctypes.data, fac.ctypes.data, ctypes.byref(h)),
              "sg_rad_tables_create")
        self._h = h
        self.chi_range = (float(xi_min), float(xi_max))
        self.nbytes = integ.nbytes + xi.nbytes + ax.nbytes


    def set_fp32_math(self, on: bool = True):
        """Monte-Carlo passes with these tables in FP32 arithmetic for the lookups, the
        optical-depth draw and the continuous loss (chi, gamma, momenta stay FP64)."""
        check(_lib.lib().sg_rad_tables_set_fp32_math(self._h, int(bool(on))), "set_fp32_math")
    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().sg_rad_tables_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def photon_chi(self, chi: torch.Tensor, xi: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(chi)
        check(_lib.lib().sg_rad_photon_chi(self._h, chi.numel(), ptr(chi), ptr(xi), ptr(out),
                                           torch.cuda.current_stream().cuda_stream), "photon_chi")
        return out

    def production_yield(self, chi: torch.Tensor, gamma: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(chi)
        check(_lib.lib().sg_rad_production_yield(self._h, chi.numel(), ptr(chi), ptr(gamma), ptr(out),
                                                 torch.cuda.current_stream().cuda_stream), "production_yield")
        return out


class PhotonChiMLP:
    """FP32 2 -> H -> H -> 1 network for log10(photon chi / chi) given log10 chi and
    log10(xi / (1 - xi)) / 3 (the inverse CDF is steep in xi at both ends)."""

    def __init__(self, hidden=64, seed=1, log10_chi_range=(-4.0, 3.0)):
        h = ctypes.c_void_p()
        check(_lib.lib().sg_mlp_create(int(hidden), int(seed), float(log10_chi_range[0]), float(log10_chi_range[1]),
                                       ctypes.byref(h)), "sg_mlp_create")
        self._h = h
        self.hidden = hidden
        n = ctypes.c_int()
        check(_lib.lib().sg_mlp_nparams(h, ctypes.byref(n)), "nparams")
        self.nparams = n.value
        self.validated = False

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().sg_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        a = np.zeros(self.nparams, dtype=np.float32)
        check(_lib.lib().sg_mlp_get_params(self._h, a.ctypes.data), "get_params")
        return a

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        check(_lib.lib().sg_mlp_set_params(self._h, a.ctypes.data), "set_params")

    def gradients(self, inputs, targets):
        X = np.ascontiguousarray(inputs, dtype=np.float32)
        T = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        l = ctypes.c_float()
        check(_lib.lib().sg_mlp_gradients(self._h, len(T), X.ctypes.data, T.ctypes.data, g.ctypes.data,
                                          ctypes.byref(l)), "gradients")
        return g, l.value

    def train(self, tables: RadiationTables, steps=2000, batch=8192, lr=2e-3, seed=7) -> float:
        l = ctypes.c_float()
        check(_lib.lib().sg_mlp_train(self._h, tables._h, int(steps), int(batch), float(lr), int(seed),
                                      ctypes.byref(l), torch.cuda.current_stream().cuda_stream), "train")
        return l.value

    def validate(self, tables: RadiationTables, n_chi_bins=28, n_xi_bins=32, per_bin=16, tol=0.02):
        err = np.zeros(n_chi_bins * n_xi_bins, dtype=np.float32)
        nm = ctypes.c_int()
        check(_lib.lib().sg_mlp_validate(self._h, tables._h, n_chi_bins, n_xi_bins, per_bin, float(tol),
                                         err.ctypes.data, ctypes.byref(nm)), "validate")
        self.validated = True
        return err.reshape(n_chi_bins, n_xi_bins), nm.value

    def photon_chi(self, chi: torch.Tensor, xi: torch.Tensor, tensor_cores: bool = True) -> torch.Tensor:
        """Batched network inverse CDF; a 64-wide network uses the tensor cores unless
        tensor_cores is False (then every layer runs on the FP32 cores)."""
        out = torch.empty_like(chi)
        fn = _lib.lib().sg_mlp_photon_chi if tensor_cores else _lib.lib().sg_mlp_photon_chi_fp32
        check(fn(self._h, chi.numel(), ptr(chi), ptr(xi), ptr(out), torch.cuda.current_stream().cuda_stream),
              "mlp photon_chi")
        return out


def monte_carlo(tables: RadiationTables, dt, mass, charge, mom, weight, tau, E, B, seed, first_id=0, step=0,
                mlp: PhotonChiMLP | None = None, chi_out=None):
    """RadiationMonteCarlo::operator() on CUDA tensors (mom[3, n], tau[n] updated in place).

    Returns (radiated energy sum w * dgamma, number of emissions)."""
    n = weight.numel()
    acc = torch.zeros(2, dtype=torch.float64, device=mom.device)
    cnt = acc[1:].view(torch.int64)
    check(_lib.lib().sg_rad_monte_carlo(tables._h, mlp._h if mlp is not None else None, n, float(dt),
                                        float(mass), float(charge), ptr(mom), ptr(weight), ptr(tau),
                                        ptr(chi_out) if chi_out is not None else None, ptr(E), ptr(B),
                                        int(seed) & 0xffffffff, int(first_id), int(step), acc.data_ptr(),
                                        acc.data_ptr() + 8, torch.cuda.current_stream().cuda_stream),
          "monte_carlo")
    torch.cuda.current_stream().synchronize()
    return float(acc[0].item()), int(cnt.item())


def monte_carlo_photons(tables: RadiationTables, dt, mass, charge, pos, mom, weight, tau, E, B, seed, first_id=0,
                        step=0, sampling=1, gamma_threshold=2.0, max_emissions=10,
                        mlp: PhotonChiMLP | None = None, chi_out=None):
    """RadiationMonteCarlo::operator() with macro-photon creation (a species whose
    radiation_photon_species is set), on CUDA tensors.  Returns (radiated energy of the
    emissions that made no photon, number of emissions, photons) where photons =
    dict(pos[ndim, k], mom[3, k], weight[k], chi[k], tau[k]) in slot order."""
    n = weight.numel()
    ndim = pos.shape[0]
    cap = max(1, n * max_emissions * sampling)
    dev = mom.device
    ph_pos = torch.empty((ndim, cap), dtype=torch.float64, device=dev)
    ph_mom = torch.empty((3, cap), dtype=torch.float64, device=dev)
    ph = torch.empty((3, cap), dtype=torch.float64, device=dev)  # weight, chi, tau
    acc = torch.zeros(3, dtype=torch.float64, device=dev)
    check(_lib.lib().sg_rad_monte_carlo_photons(
        tables._h, mlp._h if mlp is not None else None, ndim, n, float(dt), float(mass), float(charge), ptr(pos),
        ptr(mom), ptr(weight), ptr(tau), ptr(chi_out) if chi_out is not None else None, ptr(E), ptr(B),
        int(seed) & 0xffffffff, int(first_id), int(step), int(sampling), float(gamma_threshold), int(max_emissions),
        cap, ptr(ph_pos), ptr(ph_mom), ph[0].data_ptr(), ph[1].data_ptr(), ph[2].data_ptr(),
        acc.data_ptr() + 16, acc.data_ptr(), acc.data_ptr() + 8, torch.cuda.current_stream().cuda_stream),
        "monte_carlo_photons")
    torch.cuda.current_stream().synchronize()
    cnt = acc[1:].view(torch.int64)
    k = int(cnt[1].item())
    assert k <= cap
    photons = dict(pos=ph_pos[:, :k], mom=ph_mom[:, :k], weight=ph[0, :k], chi=ph[1, :k], tau=ph[2, :k])
    return float(acc[0].item()), int(cnt[0].item()), photons


def push_photons(dt, pos, mom, invgf=None):
    """PusherPhoton::operator() on CUDA tensors: pos[ndim, n] += dt p / |p| in place."""
    n = mom.shape[1]
    check(_lib.lib().sg_push_photons(pos.shape[0], n, float(dt), ptr(pos), ptr(mom),
                                     ptr(invgf) if invgf is not None else None,
                                     torch.cuda.current_stream().cuda_stream), "push_photons")
