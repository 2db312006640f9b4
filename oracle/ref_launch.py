"""Run the reference's own tcFFT kernels (cubins compiled from its source by
oracle/ref_build.sh) through the CUDA driver API.

TEST INFRASTRUCTURE ONLY: used to make parity fixtures (the reference's own
output on seeded inputs) and by the GPU parity tests when the cubins are
present. The product never loads it.

What is restated here, from yuelingfan/fft_demo:
  - the 16x16 DFT table tcfftCreate builds: F[i][j] = half(cosf(2 pi i j / 16)),
    half(-sinf(...)) (tcfft_half.cu:1332-1339, tcfft_half_2d.cu:1208-1216);
  - the launch chain of tcfftExec (tcfft_half.cu:1177-1233): layer_0[m0] over
    the whole batch, then layer_1[m_i] with step = product of earlier radices;
    block (32, 8), n_cont = {32, 16, 8}, dynamic shared memory RADIX*4*n_cont;
  - tcfftExec_2d (tcfft_half_2d.cu:1128-1149): row pass with RADIX = Ny, then
    layer_1[m1] with step = Ny, RADIX = Nx;
  - the input permutation setup()/setup_2d() apply (gen_rev), taken from the
    committed fixture tests/golden/reference_perm.npz.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
N_CONT = {0: 32, 1: 16, 2: 8}
RADIX = {0: 256, 1: 512, 2: 1024}
L0 = {0: "layer_256_0", 1: "layer_512_0", 2: "layer_1024_0"}
L1 = {0: "layer_256_1", 1: "layer_512_1"}


def mangled(base, variant, cont, with_step):
    name = base + ("_A100" if variant == "A100" else "")
    args = "iP7__half2P6__halfS3_" if with_step else "P7__half2P6__halfS3_"
    return "_Z%d%sILi%dELi8EEv%s" % (len(name), name, cont, args)


def available(kind="1d"):
    return os.path.exists(os.path.join(REF_DIR, "ref_tcfft%s.cubin" % kind))


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuInit(0)
        self.mods = {}

    def check(self, r, what):
        if r != 0:
            raise RuntimeError("CUDA driver error %d in %s" % (r, what))

    def function(self, cubin, name):
        if cubin not in self.mods:
            mod = ctypes.c_void_p()
            self.check(self.cu.cuModuleLoad(ctypes.byref(mod), cubin.encode()), "cuModuleLoad")
            self.mods[cubin] = mod
        fn = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(fn), self.mods[cubin], name.encode()),
                   "cuModuleGetFunction " + name)
        return fn

    def launch(self, fn, grid, block, smem, args):
        arr = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        self.check(self.cu.cuLaunchKernel(fn, ctypes.c_uint(grid[0]), ctypes.c_uint(grid[1]), ctypes.c_uint(1),
                                          ctypes.c_uint(block[0]), ctypes.c_uint(block[1]), ctypes.c_uint(1),
                                          ctypes.c_uint(smem), None, arr, None), "cuLaunchKernel")


_drv = None


def driver():
    global _drv
    if _drv is None:
        _drv = _Driver()
    return _drv


def dft16_tables(sign=-1):
    """F_real, F_imag as tcfftCreate builds them (FP32 cos/sin, rounded to half)."""
    i = np.arange(16, dtype=np.float32)[:, None]
    j = np.arange(16, dtype=np.float32)[None, :]
    ang = np.float32(2 * np.pi) * i * j / np.float32(16)
    fr = np.cos(ang.astype(np.float32)).astype(np.float16)
    fi = (sign * np.sin(ang.astype(np.float32))).astype(np.float16)
    return fr, fi


def run_1d(x_perm_h2, n, batch, mergings, n_mergings, variant="A100"):
    """x_perm_h2: float16 array [batch, n, 2] already in the digit-reversed
    order of setup(). Returns the reference's output (float16 [batch, n, 2])."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, "ref_tcfft1d.cubin")
    data = torch.from_numpy(np.ascontiguousarray(x_perm_h2)).cuda()
    fr, fi = dft16_tables()
    f_re = torch.from_numpy(fr.ravel().copy()).cuda()
    f_im = torch.from_numpy(fi.ravel().copy()).cuda()
    p_data = ctypes.c_void_p(data.data_ptr())
    p_fr = ctypes.c_void_p(f_re.data_ptr())
    p_fi = ctypes.c_void_p(f_im.data_ptr())
    m0 = mergings[0]
    radix, cont = RADIX[m0], N_CONT[m0]
    fn = d.function(cubin, mangled(L0[m0], variant, cont, False))
    d.launch(fn, (n * batch // cont // radix, 1), (32, 8), radix * 4 * cont, [p_data, p_fr, p_fi])
    step = radix
    for i in range(1, n_mergings):
        m = mergings[i]
        radix, cont = RADIX[m], N_CONT[m]
        fn = d.function(cubin, mangled(L1[m], variant, cont, True))
        st = ctypes.c_int(step)
        d.launch(fn, (step // cont, batch * n // step // radix), (32, 8), radix * 4 * cont,
                 [st, p_data, p_fr, p_fi])
        step *= radix
    torch.cuda.synchronize()
    return data.cpu().numpy()


def run_2d(x_perm_h2, nx, ny, batch, mergings, variant="A100"):
    """2D: x_perm_h2 float16 [batch, nx, ny, 2] permuted as setup_2d does."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, "ref_tcfft2d.cubin")
    data = torch.from_numpy(np.ascontiguousarray(x_perm_h2)).cuda()
    fr, fi = dft16_tables()
    f_re = torch.from_numpy(fr.ravel().copy()).cuda()
    f_im = torch.from_numpy(fi.ravel().copy()).cuda()
    p_data = ctypes.c_void_p(data.data_ptr())
    p_fr = ctypes.c_void_p(f_re.data_ptr())
    p_fi = ctypes.c_void_p(f_im.data_ptr())
    m0, m1 = mergings
    cont0 = N_CONT[m0]
    fn = d.function(cubin, mangled(L0[m0], variant, cont0, False))
    d.launch(fn, (nx * ny * batch // cont0 // ny, 1), (32, 8), ny * 4 * cont0, [p_data, p_fr, p_fi])
    cont1 = N_CONT[m1]
    fn = d.function(cubin, mangled(L1[m1], variant, cont1, True))
    st = ctypes.c_int(ny)
    d.launch(fn, (ny // cont1, nx * ny * batch // ny // nx), (32, 8), nx * 4 * cont1, [st, p_data, p_fr, p_fi])
    torch.cuda.synchronize()
    return data.cpu().numpy()
