"""fft_demo_gb300: tensor-core FFT / FFT convolution for one GB300 (sm_103a).

Python host mirror of the C ABI in include/tcfft_gb300.h. The compute path is
the in-tree CUDA library libtcfft_gb300.so; there is no CPU fallback: if the
library is missing or no sm_103 device is present, calls raise.

torch is used only for device memory and streams (tensors are passed to the
C ABI as raw device pointers).
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtcfft_gb300.so")

# tcfftStatus
OK, INVALID_SIZE, UNSUPPORTED, ALLOC_FAILED, LAUNCH_FAILED, TIMEOUT, CAPACITY, INVALID_VALUE, \
    NO_DEVICE = range(9)
# tcfftPrecision
FP16, SPLIT_FP32 = 0, 1
# tcfftDirection
FORWARD, INVERSE = -1, 1
# tcfftConvMode
CONV_VALID_CORR, CONV_SAME, CONV_FULL = 0, 1, 2
# tcfftBatchMode
BATCH_PERSISTENT, BATCH_PER_SIZE = 0, 1

_lib = None


class TcfftError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        name = status_string(status) if _lib is not None else str(status)
        super().__init__("%s%s" % (name, (": " + what) if what else ""))


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtcfft_gb300.so not built; run __graft_entry__.build() "
                              "or python fft_demo_gb300/build.py")
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    vp, i, ll, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
    sig = {
        "tcfft_plan_1d": (i, [ctypes.POINTER(vp), ll, ll, i]),
        "tcfft_plan_2d": (i, [ctypes.POINTER(vp), i, i, ll, i]),
        "tcfft_workspace_bytes": (i, [vp, ctypes.POINTER(ctypes.c_size_t)]),
        "tcfft_plan_set_fused": (i, [vp, i]),
        "tcfft_tune_set": (i, [i, i, i, i]),
        "tcfft_tune_prefer": (i, [i, i, i, i]),
        "tcfft_tune_get": (i, [i, i, i, ctypes.POINTER(i)]),
        "tcfft_tune_split": (i, [i, i, i]),
        "tcfft_pass_info": (i, [i, i, i, i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]),
        "tcfft_exec": (i, [vp, vp, vp, i, f, vp]),
        "tcfft_exec_digitrev": (i, [vp, vp, vp, ctypes.POINTER(i), i, vp]),
        "tcfft_exec_digitrev_2d": (i, [vp, vp, vp, ctypes.POINTER(i), i, ctypes.POINTER(i), i, i, vp]),
        "tcfft_check": (i, [vp, vp]),
        "tcfft_exec_static": (i, [vp, vp, ll, ll, i, f, vp, i]),
        "tcfft_batch_plan": (i, [ctypes.POINTER(vp), i, vp, vp, vp, vp, i, i]),
        "tcfft_batch_plan_mixed": (i, [ctypes.POINTER(vp), i, vp, vp, vp, vp, i, vp, vp, ll, i, i]),
        "tcfft_batch_exec_mixed": (i, [vp, vp, vp, vp, vp, vp]),
        "tcfft_batch_set_mode": (i, [vp, i]),
        "tcfft_queue_create": (i, [ctypes.POINTER(vp), i, ctypes.c_size_t, ctypes.c_size_t]),
        "tcfft_queue_set_filter": (i, [vp, i, vp, i, i]),
        "tcfft_queue_submit": (i, [vp, i, vp, vp, vp, vp, i, vp, vp, vp, vp, vp, vp]),
        "tcfft_queue_check": (i, [vp, vp]),
        "tcfft_queue_destroy": (i, [vp]),
        "tcfft_copy_inputs": (i, [i, vp, vp, vp, vp, vp]),
        "tcfft_batch_set_graph": (i, [vp, i]),
        "tcfft_batch_exec": (i, [vp, vp, vp, vp]),
        "tcfft_batch_info": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(i)]),
        "tcfft_batch_check": (i, [vp, vp]),
        "tcfft_batch_destroy": (i, [vp]),
        "tcfft_destroy": (i, [vp]),
        "tcfft_get_last_error": (i, []),
        "tcfft_status_string": (ctypes.c_char_p, [i]),
        "tcfft_last_launch_count": (i, []),
        "tcfft_set_wait_limit": (i, [ll]),
        "tcfft_conv2d_plan": (i, [ctypes.POINTER(vp), i, i, i, i, i, i, i, i, ll]),
        "tcfft_conv2d_set_filters": (i, [vp, vp, vp]),
        "tcfft_conv2d_set_filters_qd": (i, [vp, vp, vp]),
        "tcfft_qd_plan": (i, [ctypes.POINTER(vp), i, ll, i, i]),
        "tcfft_qd_exec": (i, [vp, vp, vp, i, vp]),
        "tcfft_qd_check": (i, [vp, vp]),
        "tcfft_qd_destroy": (i, [vp]),
        "tcfft_conv2d_exec": (i, [vp, vp, vp, ll, vp]),
        "tcfft_conv2d_shape": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]),
        "tcfft_conv2d_check": (i, [vp, vp]),
        "tcfft_conv2d_destroy": (i, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def status_string(s):
    return lib().tcfft_status_string(int(s)).decode()


def _check(status, what=""):
    if status != OK:
        raise TcfftError(status, what)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def last_launch_count():
    return lib().tcfft_last_launch_count()


def set_wait_limit(polls=-1):
    """Poll bound of the persistent kernels' dependency waits for later
    launches (tcfft_set_wait_limit); -1 restores the default, 0 makes every
    such wait give up at once (the timeout path, for tests)."""
    _check(lib().tcfft_set_wait_limit(int(polls)), "set_wait_limit")


class Plan:
    """A 1D or 2D batched C2C plan (tcfftCreate / tcfftCreate_2d equivalent).

    Data are torch tensors on the GPU: FP16 plans take interleaved complex
    half (shape [..., 2], dtype float16, or complex32 viewed as such); split
    plans take interleaved complex float32.
    """

    def __init__(self, n=None, batch=1, precision=FP16, shape2d=None):
        self._h = ctypes.c_void_p()
        self.precision = precision
        self.batch = int(batch)
        if shape2d is not None:
            nx, ny = shape2d
            self.dims, self.nx, self.ny, self.n = 2, int(nx), int(ny), int(nx) * int(ny)
            _check(lib().tcfft_plan_2d(ctypes.byref(self._h), self.nx, self.ny, self.batch,
                                       precision), "plan_2d(%d, %d, %d)" % (nx, ny, batch))
        else:
            self.dims, self.n = 1, int(n)
            _check(lib().tcfft_plan_1d(ctypes.byref(self._h), self.n, self.batch, precision),
                   "plan_1d(%d, %d)" % (n, batch))

    @property
    def elem_bytes(self):
        return 4 if self.precision == FP16 else 8

    def workspace_bytes(self):
        b = ctypes.c_size_t()
        _check(lib().tcfft_workspace_bytes(self._h, ctypes.byref(b)))
        return b.value

    def _validate(self, t):
        need = self.n * self.batch * self.elem_bytes
        if not t.is_cuda or t.numel() * t.element_size() != need or not t.is_contiguous():
            raise TcfftError(INVALID_VALUE, "tensor must be contiguous CUDA with %d bytes" % need)

    def exec(self, x, out=None, direction=FORWARD, scale=1.0, stream=None):
        """out = scale * FFT(x); out=None -> in place."""
        self._validate(x)
        if out is None:
            out = x
        self._validate(out)
        _check(lib().tcfft_exec(self._h, _ptr(x), _ptr(out), int(direction), float(scale),
                                _stream_ptr(stream)), "exec")
        return out

    def exec_digitrev(self, x, radices, out=None, stream=None):
        """Forward FFT of input in the reference's digit-reversed order."""
        self._validate(x)
        if out is None:
            out = x
        self._validate(out)
        arr = (ctypes.c_int * max(1, len(radices)))(*radices)
        _check(lib().tcfft_exec_digitrev(self._h, _ptr(x), _ptr(out), arr, len(radices),
                                         _stream_ptr(stream)), "exec_digitrev")
        return out

    def exec_digitrev_2d(self, x, radices_x, radices_y, out=None, direction=FORWARD, stream=None):
        """2D FFT of input whose axes are in the reference's digit-reversed order."""
        self._validate(x)
        if out is None:
            out = x
        self._validate(out)
        ax = (ctypes.c_int * max(1, len(radices_x)))(*radices_x)
        ay = (ctypes.c_int * max(1, len(radices_y)))(*radices_y)
        _check(lib().tcfft_exec_digitrev_2d(self._h, _ptr(x), _ptr(out), ax, len(radices_x), ay,
                                            len(radices_y), int(direction), _stream_ptr(stream)),
               "exec_digitrev_2d")
        return out

    def check(self, stream=None):
        """Synchronise and raise if a kernel of this plan flagged an error."""
        _check(lib().tcfft_check(self._h, _stream_ptr(stream)), "check")

    def set_fused(self, enable):
        """Large 1D FP16 sizes: one fused launch, or two pass launches (default)."""
        _check(lib().tcfft_plan_set_fused(self._h, 1 if enable else 0), "set_fused")

    def destroy(self):
        if self._h:
            lib().tcfft_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def exec_static(x, n, batch, out=None, direction=FORWARD, scale=1.0, stream=None, wait=True):
    """1D FP16 transform with no plan and no device allocation
    (tcfft_exec_static): 2^15 <= n <= 2^21, scratch shared by every call on
    the device, so calls that overlap on the GPU race."""
    need = int(n) * int(batch) * 4
    for t in (x,) if out is None else (x, out):
        if not t.is_cuda or t.numel() * t.element_size() != need or not t.is_contiguous():
            raise TcfftError(INVALID_VALUE, "tensor must be contiguous CUDA with %d bytes" % need)
    if out is None:
        out = x
    _check(lib().tcfft_exec_static(_ptr(x), _ptr(out), int(n), int(batch), int(direction), float(scale),
                                   _stream_ptr(stream), 1 if wait else 0), "exec_static")
    return out


class BatchConvDesc(ctypes.Structure):
    """tcfftBatchConv: one convolution of a batch plan."""
    _fields_ = [("sy", ctypes.c_int), ("sx", ctypes.c_int), ("fy", ctypes.c_int), ("fx", ctypes.c_int),
                ("mode", ctypes.c_int), ("img_off", ctypes.c_longlong), ("out_off", ctypes.c_longlong),
                ("filt_off", ctypes.c_longlong)]


def conv_output_shape(sy, sx, fy, fx, mode):
    if mode == CONV_VALID_CORR:
        return sy - fy + 1, sx - fx + 1
    if mode == CONV_SAME:
        return sy, sx
    return sy + fy - 1, sx + fx - 1


class Batch:
    """Many 1D transforms of uneven power-of-two sizes (64 <= n <= 2^20) in
    one input and one output buffer, and optionally 2D convolutions
    (tcfft_batch_plan_mixed): one persistent launch fed from a device work
    queue, or the plain per-size path.

    sizes[i], in_off[i], out_off[i]: points and element offsets of
    transform i (default: packed back to back in list order).
    convs: list of (sy, sx, fy, fx, mode) -- images, outputs and filters are
    packed back to back in list order in their own buffers; `filters` holds
    the fy x fx float filters (a CUDA float tensor or a numpy array).
    """

    def __init__(self, sizes=(), in_off=None, out_off=None, scale=None, precision=FP16, direction=FORWARD,
                 convs=(), filters=None):
        import numpy as np
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        packed = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64) if len(self.sizes) else \
            np.zeros(0, np.int64)
        self.in_off = np.ascontiguousarray(packed if in_off is None else in_off, dtype=np.int64)
        self.out_off = np.ascontiguousarray(packed if out_off is None else out_off, dtype=np.int64)
        self.scale = None if scale is None else np.ascontiguousarray(scale, dtype=np.float32)
        self.precision = precision
        self.total_in = int((self.in_off + self.sizes).max()) if len(self.sizes) else 0
        self.total_out = int((self.out_off + self.sizes).max()) if len(self.sizes) else 0
        descs = (BatchConvDesc * max(1, len(convs)))()
        img = out = filt = 0
        self.conv_shapes = []
        for k, (sy, sx, fy, fx, mode) in enumerate(convs):
            oy, ox = conv_output_shape(sy, sx, fy, fx, mode)
            descs[k] = BatchConvDesc(sy, sx, fy, fx, mode, img, out, filt)
            self.conv_shapes.append(((sy, sx), (oy, ox), img, out, filt))
            img += sy * sx
            out += oy * ox
            filt += fy * fx
        self.conv_in_elems, self.conv_out_elems, self.filter_elems = img, out, filt
        fptr = None
        if len(convs):
            if hasattr(filters, "data_ptr"):
                fptr = filters.data_ptr()
            else:
                self._filters_host = np.ascontiguousarray(filters, dtype=np.float32).ravel()
                fptr = self._filters_host.ctypes.data
        self._h = ctypes.c_void_p()
        sc = None if self.scale is None else self.scale.ctypes.data
        _check(lib().tcfft_batch_plan_mixed(
            ctypes.byref(self._h), len(self.sizes), self.sizes.ctypes.data if len(self.sizes) else None,
            self.in_off.ctypes.data if len(self.sizes) else None,
            self.out_off.ctypes.data if len(self.sizes) else None, sc, len(convs),
            ctypes.cast(descs, ctypes.c_void_p) if len(convs) else None, fptr, filt, precision, int(direction)),
            "batch_plan")

    @property
    def elem_bytes(self):
        return 4 if self.precision == FP16 else 8

    def set_mode(self, mode):
        _check(lib().tcfft_batch_set_mode(self._h, int(mode)), "batch_set_mode")

    def set_graph(self, enable):
        _check(lib().tcfft_batch_set_graph(self._h, 1 if enable else 0), "batch_set_graph")

    def info(self):
        items, ctas, ws = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        _check(lib().tcfft_batch_info(self._h, ctypes.byref(items), ctypes.byref(ws), ctypes.byref(ctas)))
        return {"items": items.value, "workspace_bytes": ws.value, "ctas": ctas.value}

    def exec(self, x=None, out=None, conv_in=None, conv_out=None, stream=None):
        rb = self.elem_bytes // 2
        checks = []
        if len(self.sizes):
            checks += [(x, self.total_in * self.elem_bytes), (out, self.total_out * self.elem_bytes)]
        if self.conv_shapes:
            checks += [(conv_in, self.conv_in_elems * rb), (conv_out, self.conv_out_elems * rb)]
        for t, need in checks:
            if t is None or not t.is_cuda or not t.is_contiguous() or t.numel() * t.element_size() < need:
                raise TcfftError(INVALID_VALUE, "tensor must be contiguous CUDA with >= %d bytes" % need)
        p = lambda t: None if t is None else _ptr(t)  # noqa: E731
        _check(lib().tcfft_batch_exec_mixed(self._h, p(x), p(out), p(conv_in), p(conv_out),
                                            _stream_ptr(stream)), "batch_exec")
        return out

    def check(self, stream=None):
        _check(lib().tcfft_batch_check(self._h, _stream_ptr(stream)), "batch_check")

    def destroy(self):
        if self._h:
            lib().tcfft_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def copy_inputs(host, src_off, nbytes, dst, dst_off, stream=None):
    """Request inputs to the device (tcfft_copy_inputs): bytes
    [src_off[i], src_off[i] + nbytes[i]) of the page-locked host tensor
    `host` to byte offset dst_off[i] of the device tensor `dst`, one
    asynchronous copy per input on `stream`."""
    import numpy as np
    src = np.ascontiguousarray(np.asarray(src_off, dtype=np.uint64) + np.uint64(host.data_ptr()))
    nb = np.ascontiguousarray(nbytes, dtype=np.uint64)
    do = np.ascontiguousarray(dst_off, dtype=np.uint64)
    if len(nb) == 0:
        return
    _check(lib().tcfft_copy_inputs(len(nb), src.ctypes.data, nb.ctypes.data, dst.data_ptr(), do.ctypes.data,
                                   _stream_ptr(stream)), "copy_inputs")


class QueueConvDesc(ctypes.Structure):
    """tcfftQueueConv: one convolution request of a queue submit."""
    _fields_ = [("sy", ctypes.c_int), ("sx", ctypes.c_int), ("filter_id", ctypes.c_int), ("mode", ctypes.c_int),
                ("img_off", ctypes.c_longlong), ("out_off", ctypes.c_longlong)]


class Queue:
    """Serving queue (tcfft_queue_*): forward 1D FFTs and convolutions with
    pooled filters, batched into one persistent launch per submit, with
    tables, filter spectra, workspace and staging resident on the device.
    One stream per queue."""

    def __init__(self, precision=FP16, workspace_bytes=1 << 30, staging_bytes=8 << 20):
        self.precision = precision
        self._h = ctypes.c_void_p()
        _check(lib().tcfft_queue_create(ctypes.byref(self._h), precision, int(workspace_bytes),
                                        int(staging_bytes)), "queue_create")

    def set_filter(self, fid, filt):
        """filt: fy x fx floats (numpy array or CUDA float tensor)."""
        import numpy as np
        if hasattr(filt, "data_ptr"):
            fy, fx = filt.shape
            ptr = filt.data_ptr()
        else:
            f = np.ascontiguousarray(filt, dtype=np.float32)
            fy, fx = f.shape
            ptr = f.ctypes.data
        _check(lib().tcfft_queue_set_filter(self._h, int(fid), ptr, int(fy), int(fx)), "queue_set_filter")

    def submit(self, n=(), in_off=(), out_off=(), convs=(), x=None, out=None, conv_in=None, conv_out=None,
               stream=None):
        """n/in_off/out_off: 1D transforms; convs: (sy, sx, filter_id, mode, img_off, out_off) tuples."""
        import numpy as np
        n = np.ascontiguousarray(n, dtype=np.int64)
        io = np.ascontiguousarray(in_off, dtype=np.int64)
        oo = np.ascontiguousarray(out_off, dtype=np.int64)
        cd = (QueueConvDesc * max(1, len(convs)))(*[QueueConvDesc(*c) for c in convs])
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        _check(lib().tcfft_queue_submit(self._h, len(n), n.ctypes.data if len(n) else None,
                                        io.ctypes.data if len(n) else None, oo.ctypes.data if len(n) else None,
                                        None, len(convs), ctypes.cast(cd, ctypes.c_void_p) if len(convs) else None,
                                        p(x), p(out), p(conv_in), p(conv_out), _stream_ptr(stream)), "queue_submit")

    def check(self, stream=None):
        _check(lib().tcfft_queue_check(self._h, _stream_ptr(stream)), "queue_check")

    def destroy(self):
        if self._h:
            lib().tcfft_queue_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def plan_1d(n, batch=1, precision=FP16):
    return Plan(n=n, batch=batch, precision=precision)


def plan_2d(nx, ny, batch=1, precision=FP16):
    return Plan(batch=batch, precision=precision, shape2d=(nx, ny))


class Conv2d:
    """2D FFT convolution plan (fft_conv2d_half / convolve_direct_fft equivalent).

    images [batch][S][sy][sx] real on the GPU (float16 for FP16 plans, float32
    for split plans); filters [F][S][fy][fx] float32 on the GPU, transformed
    once by set_filters and kept resident; exec returns [batch][F][oy][ox].
    """

    def __init__(self, S, F, sy, sx, fy, fx, mode=CONV_VALID_CORR, precision=FP16, max_batch=1):
        self._h = ctypes.c_void_p()
        self.S, self.F, self.sy, self.sx, self.fy, self.fx = S, F, sy, sx, fy, fx
        self.mode, self.precision, self.max_batch = mode, precision, max_batch
        _check(lib().tcfft_conv2d_plan(ctypes.byref(self._h), S, F, sy, sx, fy, fx, mode, precision,
                                       max_batch), "conv2d_plan")
        r, c, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().tcfft_conv2d_shape(self._h, ctypes.byref(r), ctypes.byref(c), ctypes.byref(p)))
        self.out_rows, self.out_cols, self.padded = r.value, c.value, p.value

    @property
    def dtype(self):
        import torch
        return torch.float16 if self.precision == FP16 else torch.float32

    def set_filters(self, filters, stream=None, projections=False):
        """projections=True makes the spectra by line projections
        (tcfft_conv2d_set_filters_qd) instead of the masked passes."""
        import torch
        if filters.dtype != torch.float32 or not filters.is_cuda or not filters.is_contiguous() or \
                filters.numel() != self.F * self.S * self.fy * self.fx:
            raise TcfftError(INVALID_VALUE, "filters: contiguous float32 CUDA [F][S][fy][fx]")
        self._filters = filters
        fn = lib().tcfft_conv2d_set_filters_qd if projections else lib().tcfft_conv2d_set_filters
        _check(fn(self._h, _ptr(filters), _stream_ptr(stream)), "set_filters")

    def exec(self, images, out=None, stream=None):
        import torch
        batch = images.numel() // (self.S * self.sy * self.sx)
        if images.dtype != self.dtype or not images.is_cuda or not images.is_contiguous() or \
                batch * self.S * self.sy * self.sx != images.numel():
            raise TcfftError(INVALID_VALUE, "images: contiguous %s CUDA [batch][S][sy][sx]" % self.dtype)
        if out is None:
            out = torch.empty((batch, self.F, self.out_rows, self.out_cols), dtype=self.dtype,
                              device=images.device)
        _check(lib().tcfft_conv2d_exec(self._h, _ptr(images), _ptr(out), batch, _stream_ptr(stream)),
               "conv2d_exec")
        return out

    def check(self, stream=None):
        _check(lib().tcfft_conv2d_check(self._h, _stream_ptr(stream)), "conv2d_check")

    def destroy(self):
        if self._h:
            lib().tcfft_conv2d_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class QdPlan:
    """Line-projection 2D DFT (tcfft_qd_*; the reference's qdFFT / fast_fft).

    planes: complex float32 CUDA tensor [planes][n][n][2] whose non-zeros lie
    in the top-left box_rows x box_cols box; exec returns the unnormalised 2D
    DFTs in a new tensor of the same shape.
    """

    def __init__(self, n, planes, box_rows, box_cols):
        self._h = ctypes.c_void_p()
        self.n, self.planes = int(n), int(planes)
        _check(lib().tcfft_qd_plan(ctypes.byref(self._h), self.n, self.planes, int(box_rows), int(box_cols)),
               "qd_plan")

    def exec(self, planes, out=None, direction=FORWARD, stream=None):
        import torch
        if planes.dtype != torch.float32 or not planes.is_cuda or not planes.is_contiguous() or \
                planes.numel() != self.planes * self.n * self.n * 2:
            raise TcfftError(INVALID_VALUE, "planes: contiguous float32 CUDA [planes][n][n][2]")
        if out is None:
            out = torch.empty_like(planes)
        _check(lib().tcfft_qd_exec(self._h, _ptr(planes), _ptr(out), direction, _stream_ptr(stream)), "qd_exec")
        return out

    def check(self, stream=None):
        _check(lib().tcfft_qd_check(self._h, _stream_ptr(stream)), "qd_check")

    def destroy(self):
        if self._h:
            lib().tcfft_qd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
