"""Test infrastructure: the reference's own CUDA current deposits, run on this GPU.

oracle/build_ref.sh compiles DepositCurrentDensity_3D_Order2
(src/Projector/Projector3D2OrderGPUKernelCUDAHIP.cu:136-516) and
DepositCurrentDensity_2D_Order2 (Projector2D2OrderGPUKernelCUDAHIP.cu:545-870), both
with FP64 compute and FP64 shared-memory reduction as currentDepositionKernel{3D,2D}
instantiate them, from the reference tree into oracle/_ref/ref_deposit{3,2}d.cubin
(device code only), with each kernel's entry name in ref_deposit{3,2}d.entry.  This
module loads a cubin through the CUDA driver API (libcuda via ctypes) into the primary
context torch uses and launches the kernel the way the reference's host code does: one
128-thread block per 4^D bin, grid = bins per dimension, particles sorted by bin with
bin_index[b] the end of bin b's particles.  Only tests load it; nothing in the product
path does.

Inputs follow the reference's conventions (Projector{3D,2D}2OrderGPU.cpp): positions are
the new ones, iold and deltaold describe the old ones (iold = round(x_old / dx) -
i_domain_begin, deltaold = x_old / dx - round(x_old / dx), planes [d * n + p]), and the
current arrays have the reference layout with ghosts (x-major, Jx dual in x, ...).  In
2D the out-of-plane current takes p_z and 1 / gamma.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def _files(ndim):
    return (os.path.join(HERE, "_ref", f"ref_deposit{ndim}d.cubin"),
            os.path.join(HERE, "_ref", f"ref_deposit{ndim}d.entry"))


def available(ndim: int = 3) -> bool:
    cubin, entry = _files(ndim)
    return os.path.exists(cubin) and os.path.exists(entry) and os.path.getsize(entry) > 0


class RefGpuDeposit:
    """The reference's ndim-D kernel loaded into the current device's primary context."""

    def __init__(self, ndim: int = 3, device: int = 0):
        cubin, entry = _files(ndim)
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.cu.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self._check(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.module = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.module), cubin.encode()), "cuModuleLoad")
        name = open(entry).read().strip().encode()
        self.fn = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.fn), self.module, name), "cuModuleGetFunction")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def launch(self, bins, J, J_sizes, pos, charge, weight, bin_index, invgf, iold, deltaold, inv_cell_volume,
               dx_inv, dx_ov_dt, domain_begin, nprimy, nprimz, cell_sorting=False, stream=0):
        """One launch of the 3D kernel.  bins: bins per dimension; J: three device pointers;
        pos: three device pointers (x, y, z); the other arrays device pointers; dx_inv,
        dx_ov_dt, domain_begin: three values each.  Returns immediately (stream order)."""
        vp = ctypes.c_void_p
        args = [vp(J[0]), vp(J[1]), vp(J[2]), ctypes.c_int(J_sizes[0]), ctypes.c_int(J_sizes[1]),
                ctypes.c_int(J_sizes[2]), vp(pos[0]), vp(pos[1]), vp(pos[2]), vp(charge), vp(weight),
                vp(bin_index), vp(invgf), vp(iold), vp(deltaold), ctypes.c_double(inv_cell_volume),
                ctypes.c_double(dx_inv[0]), ctypes.c_double(dx_inv[1]), ctypes.c_double(dx_inv[2]),
                ctypes.c_double(dx_ov_dt[0]), ctypes.c_double(dx_ov_dt[1]), ctypes.c_double(dx_ov_dt[2]),
                ctypes.c_int(domain_begin[0]), ctypes.c_int(domain_begin[1]), ctypes.c_int(domain_begin[2]),
                ctypes.c_int(nprimy), ctypes.c_int(nprimz), ctypes.c_int(1), ctypes.c_bool(bool(cell_sorting))]
        params = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn, int(bins[0]), int(bins[1]), int(bins[2]), 128, 1, 1, 0,
                                           ctypes.c_void_p(stream), params, None), "cuLaunchKernel")

    def launch2d(self, bins, J, J_sizes, pos, momz, charge, weight, bin_index, invgf, iold, deltaold,
                 inv_cell_volume, dx_inv, dx_ov_dt, domain_begin, nprimy, cell_sorting=False, stream=0):
        """One launch of the 2D kernel (pos: x and y device pointers, momz: p_z)."""
        vp = ctypes.c_void_p
        args = [vp(J[0]), vp(J[1]), vp(J[2]), ctypes.c_int(J_sizes[0]), ctypes.c_int(J_sizes[1]),
                ctypes.c_int(J_sizes[2]), vp(pos[0]), vp(pos[1]), vp(momz), vp(charge), vp(weight), vp(bin_index),
                vp(invgf), vp(iold), vp(deltaold), ctypes.c_double(inv_cell_volume), ctypes.c_double(dx_inv[0]),
                ctypes.c_double(dx_inv[1]), ctypes.c_double(dx_ov_dt[0]), ctypes.c_double(dx_ov_dt[1]),
                ctypes.c_int(domain_begin[0]), ctypes.c_int(domain_begin[1]), ctypes.c_int(nprimy), ctypes.c_int(1),
                ctypes.c_bool(bool(cell_sorting))]
        params = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn, int(bins[0]), int(bins[1]), 1, 128, 1, 1, 0,
                                           ctypes.c_void_p(stream), params, None), "cuLaunchKernel")
