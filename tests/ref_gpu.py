"""Launcher for the reference's own CUDA kernel (test infrastructure).

oracle/_ref/ref_kernel_sm103a.cubin is benchapps/nbody/cuda/bodysystem_kernel.cu
compiled unchanged for sm_103a (``make -C oracle ref-gpu``).  This module loads
it through the CUDA driver API and launches
_integrateNBodySystem_kernel<float> with the reference's launch shape
(benchapps/nbody/cuda/bodysystem.cu:63-79: grid N/block, ntiles = N/block,
one target per thread), so the GPU baseline can be timed beside ours.
"""
from __future__ import annotations

import ctypes as C
import os

import oracle

KERNEL_F32 = "_Z28_integrateNBodySystem_kernelIfEvPT_S1_S1_iS0_S0_S0_i"
KERNEL_F64 = "_Z28_integrateNBodySystem_kernelIdEvPT_S1_S1_iS0_S0_S0_i"


class RefKernel:
    def __init__(self):
        path = oracle.REF_CUBIN
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 6 + [C.c_uint, C.c_void_p,
                                                                            C.c_void_p, C.c_void_p]
        self.cu.cuModuleUnload.argtypes = [C.c_void_p]
        # make the device's primary context (the one the runtime and torch
        # use) current on this thread before loading the module
        self.cu.cuDevicePrimaryCtxRetain.argtypes = [C.POINTER(C.c_void_p), C.c_int]
        self.cu.cuCtxSetCurrent.argtypes = [C.c_void_p]
        dev = C.c_int()
        self._ok(self.cu.cuInit(0), "cuInit")
        self._ok(self.cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
        self.ctx = C.c_void_p()
        self._ok(self.cu.cuDevicePrimaryCtxRetain(C.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self._ok(self.cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.mod = C.c_void_p()
        self._ok(self.cu.cuModuleLoad(C.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = C.c_void_p()
        self._ok(self.cu.cuModuleGetFunction(C.byref(self.fn), self.mod, KERNEL_F32.encode()),
                 "cuModuleGetFunction")
        self.fn64 = C.c_void_p()
        self._ok(self.cu.cuModuleGetFunction(C.byref(self.fn64), self.mod, KERNEL_F64.encode()),
                 "cuModuleGetFunction")

    @staticmethod
    def _ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def step(self, pos_old, pos_new, vel, n, dt, eps2, damping, block, stream, double=False):
        """One reference step; pos/vel are device pointers (ints) of float4
        (or double4 with double=True)."""
        if n % block != 0 or block > 512:
            raise ValueError("the reference kernel needs n % block == 0 and block <= 512")
        real = C.c_double if double else C.c_float
        args = [C.c_uint64(pos_old), C.c_uint64(pos_new), C.c_uint64(vel), C.c_int(n),
                real(dt), real(eps2), real(damping), C.c_int(n // block)]
        params = (C.c_void_p * len(args))(*[C.addressof(a) for a in args])
        fn = self.fn64 if double else self.fn
        # the kernel's shared tile is 4 T per thread (sharedPos[4][512] of T)
        self._ok(self.cu.cuLaunchKernel(fn, n // block, 1, 1, block, 1, 1, 0,
                                        C.c_void_p(stream), params, None), "cuLaunchKernel")

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None
