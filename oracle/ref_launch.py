"""Run the reference's own tcFFT and FFT-convolution kernels (cubins compiled
from its source by oracle/ref_build.sh) through the CUDA driver API.

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
    committed fixture tests/golden/reference_perm.npz;
  - fft_conv2d_half's forward convolution (tensorcore_fft_conv2d.cpp:12-58
    constructor, :250-289 TENSORCORE_FFT_CONV_2D / readout_fwd;
    tensorcore_fft_conv2d_kernel.cu:1101-1150 fft_pointwise and
    fft_conv_final_stage, :1255-1275 fft_conv2d_inv_rev_pad, :1399
    read_out_scale_double2double, :1495-1525 TensorCoreFFTExec) with its
    _A100 kernel wiring (:1565-1571), in run_conv_valid.
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


# ---------------------------------------------------------------------------
# fft_conv2d_half::conv2d_forward (valid cross-correlation), reference kernels
# ---------------------------------------------------------------------------
CONV_CUBIN = "ref_conv.cubin"
_CONV_K = {
    "inv": "_Z25fft_conv2d_inverse_filterPdii",
    "inv_odd": "_Z29fft_conv2d_inverse_filter_oddPdii",
    "pad": "_Z46fft_conv2d_bit_rev_real_pad_to_cpx_double2halfPdP6__halfPiS2_iiii",
    "mul_add": "_Z26fft_cpx_point_wise_mul_addP6__halfS0_Pfiiii",
    "q1": "_Z27fft_cpx_point_wise_quant_p1PfS_ii",
    "q2": "_Z27fft_cpx_point_wise_quant_p2PfS_ii",
    "q3": "_Z27fft_cpx_point_wise_quant_p3PfP6__halfS_PiS2_ii",
    "deq": "_Z26fft_cpx_point_wise_dequantP6__halfPdPfii",
    "read": "_Z35read_out_scale_double2double_kernelPdS_iiiiid",
}


def conv_available():
    return os.path.exists(os.path.join(REF_DIR, CONV_CUBIN))


def _conv_stage(base, m, with_step):
    cont = N_CONT[m]
    name = base + "_A100"
    args = "iP7__half2P6__halfS3_i" if with_step else "P7__half2P6__halfS3_i"
    return "_Z%d%sILi%dELi8EEv%s" % (len(name), name, cont, args)


def _tc_exec_2d(d, cubin, data, P, batch, fft):
    """TensorCoreFFTExec (kernel.cu:1526-1555) of a P x P plan, fft = +-1."""
    import torch
    m = {256: 0, 512: 1}[P]
    fr, fi = dft16_tables(sign=-1 if fft == 1 else 1)
    f_re = torch.from_numpy(fr.ravel().copy()).cuda()
    f_im = torch.from_numpy(fi.ravel().copy()).cuda()
    p_data = ctypes.c_void_p(data.data_ptr())
    p_fr, p_fi = ctypes.c_void_p(f_re.data_ptr()), ctypes.c_void_p(f_im.data_ptr())
    cont = N_CONT[m]
    fn = d.function(cubin, _conv_stage(L0[m], m, False))
    d.launch(fn, (P * P * batch // cont // P, 1), (32, 8), P * 4 * cont, [p_data, p_fr, p_fi, ctypes.c_int(fft)])
    fn = d.function(cubin, _conv_stage(L1[m], m, True))
    d.launch(fn, (P // cont, P * P * batch // P // P), (32, 8), P * 4 * cont,
             [ctypes.c_int(P), p_data, p_fr, p_fi, ctypes.c_int(fft)])
    torch.cuda.synchronize()


def run_conv_valid(signal, filters, rev_tables):
    """The reference's fft_conv2d_half(signal, filter, S, F, sy, sx, fy, fx,
    __AMPERE__) followed by conv2d_forward(output).
    signal [S][sy][sx], filters [F][S][fy][fx] (float64); rev_tables: {256:
    rev_256, 512: rev_512} (the header's tables, tests/golden/
    reference_perm.npz). Returns output [F][sy-fy+1][sx-fx+1] (float64).
    One deviation, for determinism: the FP32 pointwise buffer is zeroed before
    fft_cpx_point_wise_mul_add accumulates into it (the reference accumulates
    into a fresh cudaMalloc, kernel.cu:1107)."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, CONV_CUBIN)
    S, sy, sx = signal.shape
    F, S2, fy, fx = filters.shape
    assert S == S2
    P = 256 if sx + fx - 1 <= 256 else 512
    oy, ox = sy - fy + 1, sx - fx + 1
    dev = torch.device("cuda")
    cu_signal = torch.from_numpy(np.ascontiguousarray(signal, dtype=np.float64)).to(dev)
    cu_filter = torch.from_numpy(np.ascontiguousarray(filters, dtype=np.float64)).to(dev)
    sig_pad = torch.zeros(S * P * P * 2, dtype=torch.float16, device=dev)
    filt_pad = torch.zeros(F * S * P * P * 2, dtype=torch.float16, device=dev)
    rev = torch.zeros(1024, dtype=torch.int32, device=dev)
    rev[:P] = torch.from_numpy(np.asarray(rev_tables[P], dtype=np.int32))
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    I = ctypes.c_int  # noqa: E741
    fn = lambda k: d.function(cubin, _CONV_K[k])  # noqa: E731
    # fft_conv2d_inv_rev_pad (kernel.cu:1255): rotate the filters in place, pad
    d.launch(fn("inv"), (F * S, fy // 2), (fx, 1), 0, [ptr(cu_filter), I(fx), I(fy)])
    if fy & 1 and fx // 2 > 0:
        d.launch(fn("inv_odd"), (F * S, 1), (fx // 2, 1), 0, [ptr(cu_filter), I(fx), I(fy)])
    d.launch(fn("pad"), (S, P), (P, 1), 0, [ptr(cu_signal), ptr(sig_pad), ptr(rev), ptr(rev), I(P), I(P), I(sx), I(sy)])
    d.launch(fn("pad"), (F * S, P), (P, 1), 0,
             [ptr(cu_filter), ptr(filt_pad), ptr(rev), ptr(rev), I(P), I(P), I(fx), I(fy)])
    torch.cuda.synchronize()
    _tc_exec_2d(d, cubin, sig_pad, P, S, 1)
    _tc_exec_2d(d, cubin, filt_pad, P, F * S, 1)
    # fft_pointwise (kernel.cu:1101): FP32 sum over channels, per-filter
    # power-of-ten quantisation, digit-reversed FP16 planes
    pw_f = torch.zeros(F * P * P * 2, dtype=torch.float32, device=dev)
    pw_h = torch.zeros(F * P * P * 2, dtype=torch.float16, device=dev)
    max_line = torch.zeros(F * P, dtype=torch.float32, device=dev)
    max_tile = torch.zeros(F, dtype=torch.float32, device=dev)
    d.launch(fn("mul_add"), (F, P), (P, 1), 0, [ptr(sig_pad), ptr(filt_pad), ptr(pw_f), I(S), I(F), I(P), I(P)])
    d.launch(fn("q1"), (F, 1), (P, 1), 0, [ptr(pw_f), ptr(max_line), I(P), I(P)])
    d.launch(fn("q2"), (1, 1), (F, 1), 0, [ptr(max_line), ptr(max_tile), I(P), I(P)])
    d.launch(fn("q3"), (F, P), (P, 1), 0, [ptr(pw_f), ptr(pw_h), ptr(max_tile), ptr(rev), ptr(rev), I(P), I(P)])
    torch.cuda.synchronize()
    _tc_exec_2d(d, cubin, pw_h, P, F, -1)
    # fft_conv_final_stage (kernel.cu:1141) and readout_fwd (.cpp:275)
    padded = torch.zeros(F * P * P * 2, dtype=torch.float64, device=dev)
    d.launch(fn("deq"), (F, P), (P, 1), 0, [ptr(pw_h), ptr(padded), ptr(max_tile), I(P), I(P)])
    out = torch.zeros(F * oy * ox, dtype=torch.float64, device=dev)
    scale = float(np.float32(1.0) / np.float32(P * P))
    d.launch(fn("read"), (F, oy), (ox, 1), 0,
             [ptr(padded), ptr(out), I(P), I(P), I(ox), I(oy), I(fx), ctypes.c_double(scale)])
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(F, oy, ox)


# ---------------------------------------------------------------------------
# Timing of the reference's own GPU kernels (the bench's reference arm)
# ---------------------------------------------------------------------------
def _events_ms(fn, reps=20, warm=3):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def time_1d(n, batch, reps=20):
    """ms per tcfftExec (tcfft_half.cu:1177) of the _A100 wiring for the one-
    launch sizes (256, 512, 1024), batch sequences."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, "ref_tcfft1d.cubin")
    m0 = {256: 0, 512: 1, 1024: 2}[n]
    data = (torch.rand(batch * n * 2, device="cuda") * 2 - 1).half()
    fr, fi = dft16_tables()
    f_re = torch.from_numpy(fr.ravel().copy()).cuda()
    f_im = torch.from_numpy(fi.ravel().copy()).cuda()
    args = [ctypes.c_void_p(data.data_ptr()), ctypes.c_void_p(f_re.data_ptr()), ctypes.c_void_p(f_im.data_ptr())]
    fn = d.function(cubin, mangled(L0[m0], "A100", N_CONT[m0], False))
    cont = N_CONT[m0]
    return _events_ms(lambda: d.launch(fn, (n * batch // cont // RADIX[m0], 1), (32, 8), RADIX[m0] * 4 * cont, args),
                      reps)


def time_2d(n, batch, reps=20):
    """ms per tcfftExec_2d (tcfft_half_2d.cu:1128) of an n x n plan (256 or 512)."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, "ref_tcfft2d.cubin")
    m = {256: 0, 512: 1}[n]
    data = (torch.rand(batch * n * n * 2, device="cuda") * 2 - 1).half()
    fr, fi = dft16_tables()
    f_re = torch.from_numpy(fr.ravel().copy()).cuda()
    f_im = torch.from_numpy(fi.ravel().copy()).cuda()
    p = [ctypes.c_void_p(data.data_ptr()), ctypes.c_void_p(f_re.data_ptr()), ctypes.c_void_p(f_im.data_ptr())]
    f0 = d.function(cubin, mangled(L0[m], "A100", N_CONT[m], False))
    f1 = d.function(cubin, mangled(L1[m], "A100", N_CONT[m], True))
    cont = N_CONT[m]

    def run():
        d.launch(f0, (n * n * batch // cont // n, 1), (32, 8), n * 4 * cont, p)
        d.launch(f1, (n // cont, n * n * batch // n // n), (32, 8), n * 4 * cont, [ctypes.c_int(n)] + p)

    return _events_ms(run, reps)


def time_conv_valid(S, F, side, f, rev_tables, reps=10):
    """ms per fft_conv2d_half(signal, filter, ...) + conv2d_forward(output)
    on the device: the constructor's flip, pad and two forward transforms
    (the reference transforms its filters on every construction), the
    pointwise product, quantisation, inverse transform, dequantisation and
    read-out -- the launch sequence of run_conv_valid, without its host
    allocations, copies and synchronisations."""
    import torch
    d = driver()
    cubin = os.path.join(REF_DIR, CONV_CUBIN)
    P = 256 if side + f - 1 <= 256 else 512
    oy = side - f + 1
    dev = torch.device("cuda")
    cu_signal = torch.rand(S * side * side, dtype=torch.float64, device=dev)
    cu_filter = torch.rand(F * S * f * f, dtype=torch.float64, device=dev)
    sig_pad = torch.zeros(S * P * P * 2, dtype=torch.float16, device=dev)
    filt_pad = torch.zeros(F * S * P * P * 2, dtype=torch.float16, device=dev)
    rev = torch.zeros(1024, dtype=torch.int32, device=dev)
    rev[:P] = torch.from_numpy(np.asarray(rev_tables[P], dtype=np.int32))
    pw_f = torch.zeros(F * P * P * 2, dtype=torch.float32, device=dev)
    pw_h = torch.zeros(F * P * P * 2, dtype=torch.float16, device=dev)
    max_line = torch.zeros(F * P, dtype=torch.float32, device=dev)
    max_tile = torch.zeros(F, dtype=torch.float32, device=dev)
    padded = torch.zeros(F * P * P * 2, dtype=torch.float64, device=dev)
    out = torch.zeros(F * oy * oy, dtype=torch.float64, device=dev)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    I = ctypes.c_int  # noqa: E741
    k = {name: d.function(cubin, sym) for name, sym in _CONV_K.items()}
    m = {256: 0, 512: 1}[P]
    cont = N_CONT[m]
    stage = {}
    tables = {}
    for fft in (1, -1):
        fr, fi = dft16_tables(sign=-1 if fft == 1 else 1)
        tables[fft] = (torch.from_numpy(fr.ravel().copy()).cuda(), torch.from_numpy(fi.ravel().copy()).cuda())
        stage[fft] = (d.function(cubin, _conv_stage(L0[m], m, False)), d.function(cubin, _conv_stage(L1[m], m, True)))

    def exec2d(t, batch, fft):
        f0, f1 = stage[fft]
        fr, fi = tables[fft]
        p = [ptr(t), ptr(fr), ptr(fi)]
        d.launch(f0, (P * P * batch // cont // P, 1), (32, 8), P * 4 * cont, p + [I(fft)])
        d.launch(f1, (P // cont, batch), (32, 8), P * 4 * cont, [I(P)] + p + [I(fft)])

    scale = float(np.float32(1.0) / np.float32(P * P))

    def run():
        d.launch(k["inv"], (F * S, f // 2), (f, 1), 0, [ptr(cu_filter), I(f), I(f)])
        if f & 1 and f // 2 > 0:
            d.launch(k["inv_odd"], (F * S, 1), (f // 2, 1), 0, [ptr(cu_filter), I(f), I(f)])
        d.launch(k["pad"], (S, P), (P, 1), 0, [ptr(cu_signal), ptr(sig_pad), ptr(rev), ptr(rev), I(P), I(P), I(side),
                                                I(side)])
        d.launch(k["pad"], (F * S, P), (P, 1), 0, [ptr(cu_filter), ptr(filt_pad), ptr(rev), ptr(rev), I(P), I(P),
                                                    I(f), I(f)])
        exec2d(sig_pad, S, 1)
        exec2d(filt_pad, F * S, 1)
        d.launch(k["mul_add"], (F, P), (P, 1), 0, [ptr(sig_pad), ptr(filt_pad), ptr(pw_f), I(S), I(F), I(P), I(P)])
        d.launch(k["q1"], (F, 1), (P, 1), 0, [ptr(pw_f), ptr(max_line), I(P), I(P)])
        d.launch(k["q2"], (1, 1), (F, 1), 0, [ptr(max_line), ptr(max_tile), I(P), I(P)])
        d.launch(k["q3"], (F, P), (P, 1), 0, [ptr(pw_f), ptr(pw_h), ptr(max_tile), ptr(rev), ptr(rev), I(P), I(P)])
        exec2d(pw_h, F, -1)
        d.launch(k["deq"], (F, P), (P, 1), 0, [ptr(pw_h), ptr(padded), ptr(max_tile), I(P), I(P)])
        d.launch(k["read"], (F, oy), (oy, 1), 0, [ptr(padded), ptr(out), I(P), I(P), I(oy), I(oy), I(f),
                                                   ctypes.c_double(scale)])

    return _events_ms(run, reps)
