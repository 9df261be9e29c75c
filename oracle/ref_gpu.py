"""The reference's own CUDA fitter kernels on this GPU (baseline and test
infrastructure only, never the product path).

kernel_bsplineMLEFit_z_EMCCD / _4D_EMCCD / _5n3D_EMCCD
(MultiD_bspline/visual code/GPUmleFit_LM/GPUmleFit_LM_EMCCD.cu:1208-2405) are
compiled from the reference sources by oracle/build_ref.sh into
oracle/_ref/ref_emccd.ptx and launched here through the CUDA driver API the way
the reference mex launches them (GPUmleFit_LM/mexFunction.cpp:598-674,
wrapper.cu:256-279): one thread per ROI, 64 threads per block
(definitions.h:10, mexFunction.cpp:407), nData = size - 3 per axis, `deg` and
`temp` null (unused by the kernels), initP in device memory for fit types 7 and
8. These are the reference's GPU variants, which differ from its CPU fitter in
the places listed for the GPU-vs-CPU divergences (x/y swapped in fit type 6's
initial and CRLB passes, other clamps and bounds in 7 and 8); the product and
the oracle follow the CPU fitter.

The coefficient table is copied into a buffer with one outermost-axis stride of
zeros after it: the derivative's +1 neighbour of a position exactly on the last
knot reads one node past its axis, and the padding keeps that read inside the
allocation.
"""
import ctypes
import os

import numpy as np

from .build import REF_DIR

PTX = os.path.join(REF_DIR, "ref_emccd.ptx")
NAMES = {6: "kernel_bsplineMLEFit_z_EMCCD", 7: "kernel_bsplineMLEFit_4D_EMCCD",
         8: "kernel_bsplineMLEFit_5n3D_EMCCD"}
NV = {6: 5, 7: 6, 8: 8}
BLOCK = 64


def available():
    return os.path.exists(PTX)


class RefGPU:
    def __init__(self):
        import torch
        if not available():
            raise RuntimeError(f"{PTX} is not built (oracle/build_ref.sh)")
        torch.zeros(1, device="cuda")  # the runtime's primary context, current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        self._img = ctypes.create_string_buffer(open(PTX, "rb").read() + b"\0")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoadData(ctypes.byref(self.mod), self._img), "cuModuleLoadData")
        n = ctypes.c_uint()
        self._check(self.cu.cuModuleGetFunctionCount(ctypes.byref(n), self.mod),
                    "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * n.value)()
        self._check(self.cu.cuModuleEnumerateFunctions(funcs, n, self.mod),
                    "cuModuleEnumerateFunctions")
        self.fn = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._check(self.cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)),
                        "cuFuncGetName")
            nm = name.value.decode()
            for ft, base in NAMES.items():
                if f"{len(base)}{base}P" in nm:  # the mangled name's first parameter follows
                    self.fn[ft] = ctypes.c_void_p(f)
        missing = [ft for ft in NAMES if ft not in self.fn]
        if missing:
            raise RuntimeError(f"reference kernels not found for fit types {missing}")

    def _check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value})")

    @staticmethod
    def padded_table(coeff, device):
        """Device copy of a C-order coefficient array with one outermost
        stride of zeros after it."""
        import torch
        c = np.ascontiguousarray(coeff, dtype=np.float32).ravel()
        pad = int(np.prod(coeff.shape[1:])) if coeff.ndim > 1 else 1
        t = torch.zeros(c.size + pad, dtype=torch.float32, device=device)
        t[: c.size] = torch.from_numpy(c).to(device)
        return t

    def fit(self, fittype, rois, iterations, d_coeff, dims, d_coeff3=None, d_initp=None,
            stream=None, out=None):
        """Launch the reference kernel of `fittype` on device tensors.
        rois: float32 (N, s, s); d_coeff: padded_table(); dims: the MATLAB
        sizes of the coefficient array (fastest first). Returns (P, CRLB, LL)
        device tensors in the reference's column-major layout."""
        import torch
        n, s = int(rois.shape[0]), int(rois.shape[-1])
        nv = NV[fittype]
        if out is None:
            P = torch.empty(((nv + 1) * n,), dtype=torch.float32, device=rois.device)
            C = torch.empty((nv * n,), dtype=torch.float32, device=rois.device)
            L = torch.empty((n,), dtype=torch.float32, device=rois.device)
        else:
            P, C, L = out
        nd = [int(d) - 3 for d in dims]
        vp = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None else 0)  # noqa: E731
        args = [vp(rois), vp(d_coeff)]
        if fittype == 8:
            args.append(vp(d_coeff3))
        args += [ctypes.c_int(x) for x in nd]
        args += [ctypes.c_int(s), ctypes.c_int(int(iterations))]
        if fittype in (7, 8):
            args.append(vp(d_initp))
        args += [vp(P), vp(C), vp(L), ctypes.c_int(n), ctypes.c_void_p(0)]
        if fittype == 6:
            args.append(ctypes.c_void_p(0))
        params = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        grid = (n + BLOCK - 1) // BLOCK
        if n > 0:
            self._check(self.cu.cuLaunchKernel(self.fn[fittype], grid, 1, 1, BLOCK, 1, 1, 0,
                                               ctypes.c_void_p(st.cuda_stream), params, None),
                        "cuLaunchKernel")
        return P, C, L
