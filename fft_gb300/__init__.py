"""afft_gb300: GB300 power-of-two FFTs behind afft's C API.

The product is ``libafft_gb300.so`` (CUDA kernels + C ABI, see
include/afft_gb300.h).  This module is its Python front end: ctypes bindings
of every exported entry point, and classes that mirror afft's C++ wrapper
fft.hpp (``complex_transform``, ``inverse_complex_transform``,
``real_transform``, ``inverse_real_transform``; fft.hpp:48-234) with the same
construction arguments and call signatures, plus ``BatchPlan`` and ``Queue``
for the batched and multi-transform extensions.

Arrays may be torch CUDA tensors (device pointers: the transform runs on
device memory) or numpy arrays / CPU tensors (host pointers: the library
stages the data through device buffers).  There is no CPU fallback: if the
library cannot be loaded, importing this module raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libafft_gb300.so")

# fft.h:5-15 and the extension enums of include/afft_gb300.h
afft_auto, afft_scalar, afft_sse2, afft_avx2, afft_avx512f, afft_neon, afft_gb300 = range(7)
afft_split, afft_interleaved = 0, 1
KIND_C, KIND_CI, KIND_R, KIND_RI = 0, 1, 2, 3
FORM_TC = 0x100   # AFFT_GB300_FORM_TC: split-precision tensor-core butterflies
FORM_F64 = 0x200  # AFFT_GB300_FORM_F64: FP64 data and arithmetic (the afft_64_* path)
QUEUE_TUNED = 0x400  # AFFT_GB300_QUEUE_TUNED: queue plans take the autotuner's per-shape choices
KINDS = {"c": KIND_C, "ci": KIND_CI, "r": KIND_R, "ri": KIND_RI}
ERRORS = {0: "OK", 1: "EINVAL", 2: "ENODEV", 3: "ENOMEM", 4: "ECUDA", 5: "ESTATE", 6: "ETIMEOUT"}

_lib = None


class AfftError(RuntimeError):
    pass


class Desc(ctypes.Structure):
    """afft_gb300_desc"""
    _fields_ = [("kind", ctypes.c_int), ("ndim", ctypes.c_int), ("dim", ctypes.c_size_t * 3),
                ("src_re", ctypes.c_void_p), ("src_im", ctypes.c_void_p),
                ("dst_re", ctypes.c_void_p), ("dst_im", ctypes.c_void_p)]


def lib():
    """The loaded CUDA library.  Raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libafft_gb300.so is not built; run `python -m fft_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        S, P, I = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        for k in ("c", "ci", "r", "ri"):
            for bits in ("32", "64"):
                ms = getattr(L, "afft_%s_%s_memsize" % (bits, k))
                ms.restype = S
                ms.argtypes = [S, P, I, I]
                cr = getattr(L, "afft_%s_%s_create" % (bits, k))
                cr.restype = P
                cr.argtypes = [S, P, I, P, I]
                tr = getattr(L, "afft_%s_%s_transform" % (bits, k))
                tr.restype = None
                tr.argtypes = [P, P, P, P, P] if k in ("c", "ci") else [P, P, P, P]
        L.afft_32_align_size.restype = S
        L.afft_32_align_size.argtypes = [S]
        L.afft_64_align_size.restype = S
        L.afft_64_align_size.argtypes = [S]
        L.afft_supported.restype = I
        L.afft_supported.argtypes = [I]
        L.afft_gb300_last_error.restype = I
        L.afft_gb300_last_error_string.restype = ctypes.c_char_p
        L.afft_gb300_batch_memsize.restype = S
        L.afft_gb300_batch_memsize.argtypes = [I, S, P, S, I]
        L.afft_gb300_batch_create.restype = P
        L.afft_gb300_batch_create.argtypes = [I, S, P, S, I, P]
        L.afft_gb300_transform_async.restype = I
        L.afft_gb300_transform_async.argtypes = [P, P, P, P, P, P]
        L.afft_gb300_release.restype = I
        L.afft_gb300_release.argtypes = [P]
        L.afft_gb300_plan_launches.restype = I
        L.afft_gb300_plan_launches.argtypes = [P]
        L.afft_gb300_queue_create.restype = P
        L.afft_gb300_queue_create.argtypes = [P, S]
        L.afft_gb300_queue_create_ex.restype = P
        L.afft_gb300_queue_create_ex.argtypes = [P, S, I]
        L.afft_gb300_plan_describe.restype = S
        L.afft_gb300_plan_describe.argtypes = [I, S, P, S, I, ctypes.c_char_p, S]
        L.afft_gb300_tune.restype = I
        L.afft_gb300_tune.argtypes = [I, S, P, S, I, ctypes.c_char_p, S]
        L.afft_gb300_tuned.restype = I
        L.afft_gb300_tuned.argtypes = [I, S, P, S, I, P, P]
        L.afft_gb300_c2c_noalloc.restype = I
        L.afft_gb300_c2c_noalloc.argtypes = [P, P, P, P, S, S, I, P]
        L.afft_gb300_queue_run.restype = I
        L.afft_gb300_queue_run.argtypes = [P, P]
        L.afft_gb300_queue_launches.restype = I
        L.afft_gb300_queue_launches.argtypes = [P]
        L.afft_gb300_queue_destroy.restype = None
        L.afft_gb300_queue_destroy.argtypes = [P]
        _lib = L
    return _lib


def last_error():
    L = lib()
    return L.afft_gb300_last_error(), L.afft_gb300_last_error_string().decode()


def _check(what):
    code, msg = last_error()
    if code:
        raise AfftError("%s: %s (%s)" % (what, msg, ERRORS.get(code, code)))


def alignment():
    return ctypes.c_size_t.in_dll(lib(), "afft_alignment").value


def align_size(n):
    return lib().afft_32_align_size(n)


def supported(impl=afft_auto):
    return bool(lib().afft_supported(impl))


def ptr(a):
    """Address of a torch tensor, numpy array or int (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if hasattr(a, "ctypes"):
        return a.ctypes.data
    raise TypeError(type(a))


def _validate(kind, dims, batch, fmt, bits, src_re, src_im, dst_re, dst_im):
    """Check the array objects a transform call gets (numpy arrays, torch
    tensors): element type, contiguity and size against what the transform
    reads and writes, so that a wrong array is refused here instead of the
    kernels reading or writing past it.  Raw int pointers are not checked."""
    k = KINDS[kind] if isinstance(kind, str) else kind
    d = squeeze(dims)
    n = 1
    for x in d:
        n *= x
    h = half_elems(d)
    inter = fmt == afft_interleaved
    cin, cout = k != KIND_R, k != KIND_RI
    m_in = (h if k == KIND_RI else n) * batch
    m_out = (h if k == KIND_R else n) * batch
    want = {"src_re": m_in * (2 if cin and inter else 1), "src_im": m_in if cin and not inter else 0,
            "dst_re": m_out * (2 if cout and inter else 1), "dst_im": m_out if cout and not inter else 0}
    name = "float64" if bits == 64 else "float32"
    for role, a in (("src_re", src_re), ("src_im", src_im), ("dst_re", dst_re), ("dst_im", dst_im)):
        if a is None or isinstance(a, int) or not want[role] or not hasattr(a, "dtype"):
            continue
        if str(a.dtype).split(".")[-1] != name:
            raise AfftError("%s: %s array expected, got %s" % (role, name, a.dtype))
        size = a.numel() if hasattr(a, "numel") else a.size
        contig = a.is_contiguous() if hasattr(a, "is_contiguous") else a.flags["C_CONTIGUOUS"]
        if not contig:
            raise AfftError("%s: the array must be contiguous" % role)
        if size < want[role]:
            raise AfftError("%s: %d elements, the transform needs %d" % (role, size, want[role]))


def describe(kind, dims, batch=1, fmt=0):
    """The kernel launches a batched plan issues, as a dict (from
    afft_gb300_plan_describe; no device needed)."""
    import json
    L = lib()
    k = KINDS[kind] if isinstance(kind, str) else kind
    arr, n = _dims(dims)
    size = L.afft_gb300_plan_describe(k, n, arr, batch, fmt, None, 0)
    if size == 0:
        _check("plan_describe")
        raise AfftError("plan_describe rejected the plan")
    buf = ctypes.create_string_buffer(size)
    L.afft_gb300_plan_describe(k, n, arr, batch, fmt, buf, size)
    return json.loads(buf.value.decode())


def tune(kind, dims, batch=1, fmt=afft_split):
    """Run the autotuner for a shape on the current device (afft_gb300_tune);
    returns its report: the candidates with median times and the choice."""
    import json
    L = lib()
    k = KINDS[kind] if isinstance(kind, str) else kind
    arr, n = _dims(dims)
    buf = ctypes.create_string_buffer(65536)
    if L.afft_gb300_tune(k, n, arr, batch, fmt, buf, len(buf)):
        _check("tune")
        raise AfftError("tune failed")
    return json.loads(buf.value.decode())


def tuned(kind, dims, batch=1, fmt=afft_split):
    """The autotuner's choice for a shape, {"split", "real_inv"}, or None."""
    L = lib()
    k = KINDS[kind] if isinstance(kind, str) else kind
    arr, n = _dims(dims)
    a, b = ctypes.c_int(), ctypes.c_int()
    r = L.afft_gb300_tuned(k, n, arr, batch, fmt, ctypes.byref(a), ctypes.byref(b))
    if r < 0:
        _check("tuned")
        raise AfftError("bad shape")
    return {"split": a.value, "real_inv": b.value} if r == 1 else None


def pass_bytes(desc):
    """Bytes the launches of a described plan must move between them: one
    read of each launch's input and one write of its output (split FP32,
    8 bytes per complex element), summed over launches."""
    total = 0
    for op in desc["ops"]:
        t = op["type"]
        if t == "line":
            L, n, lk = 1 << op["logl"], op["nlines"], op["lk"]
            if lk in (1, 2):          # real forward / inverse: L complex one way, L + 1 the other
                total += n * 8 * (2 * L + 1)
            else:                     # complex, and the paired real passes of long 1D axes
                total += n * 16 * L
        elif t == "real":
            total += op["nlines"] * 8 * (2 * op["L"] + 1)
        elif t == "copy":
            total += op["nlines"] * 16 * op["len"]
        else:                         # length-1 real transforms
            total += op["nlines"] * 12
    return total


def _dims(dims):
    dims = [int(d) for d in dims]
    return (ctypes.c_size_t * max(1, len(dims)))(*dims), len(dims)


def squeeze(dims):
    d = [int(x) for x in dims if int(x) != 1]
    return d or [1]


def half_elems(dims):
    """Elements per array of a real transform's half spectrum (dim 0 halved,
    fft_internal.hpp:215-219 without the alignment padding)."""
    d = squeeze(dims)
    n = 1
    for x in d[1:]:
        n *= x
    return (d[0] // 2 + 1) * n


class _Plan:
    """A plan placement-built into caller-owned memory (fft.hpp:8-47).
    ``bits`` selects the afft_32_* (float) or afft_64_* (double) entry points,
    as fft.hpp's class templates do for T = float / double."""

    kind = None

    def __init__(self, dims, mem=None, impl=afft_auto, fmt=afft_split, bits=32):
        L = lib()
        if bits not in (32, 64):
            raise ValueError("bits must be 32 or 64")
        self.dims = [int(d) for d in dims]
        self.format = fmt
        self.bits = bits
        arr, n = _dims(self.dims)
        name = {KIND_C: "c", KIND_CI: "ci", KIND_R: "r", KIND_RI: "ri"}[self.kind]
        size = getattr(L, "afft_%d_%s_memsize" % (bits, name))(n, arr, fmt, impl)
        self._mem = None
        self.state = None
        if size == 0 or size == ctypes.c_size_t(-1).value:
            _check("memsize")
            raise AfftError("memsize rejected the plan")
        self._mem = mem if mem is not None else ctypes.create_string_buffer(size)
        self.state = getattr(L, "afft_%d_%s_create" % (bits, name))(n, arr, fmt, ctypes.addressof(self._mem), impl)
        if not self.state:
            _check("create")
            raise AfftError("create failed")
        self._fn = getattr(L, "afft_%d_%s_transform" % (bits, name))

    def __bool__(self):
        return bool(self.state)

    def release(self):
        if self.state:
            lib().afft_gb300_release(self.state)
            self.state = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @property
    def launches(self):
        return lib().afft_gb300_plan_launches(self.state)


class complex_transform(_Plan):
    """fft.hpp:48-95: forward complex transform, split or interleaved."""
    kind = KIND_C

    def __call__(self, src_re, src_im, dst_re, dst_im):
        _validate(self.kind, self.dims, 1, self.format, self.bits, src_re, src_im, dst_re, dst_im)
        self._fn(self.state, ptr(src_re), ptr(src_im), ptr(dst_re), ptr(dst_im))
        _check("transform")


class inverse_complex_transform(complex_transform):
    """fft.hpp:97-144: unnormalised inverse complex transform."""
    kind = KIND_CI


class real_transform(_Plan):
    """fft.hpp:146-189: real forward transform, first dim halved."""
    kind = KIND_R

    def __call__(self, src, dst_re, dst_im):
        _validate(self.kind, self.dims, 1, self.format, self.bits, src, None, dst_re, dst_im)
        self._fn(self.state, ptr(src), ptr(dst_re), ptr(dst_im))
        _check("transform")


class inverse_real_transform(_Plan):
    """fft.hpp:191-234: unnormalised real inverse transform."""
    kind = KIND_RI

    def __call__(self, src_re, src_im, dst):
        _validate(self.kind, self.dims, 1, self.format, self.bits, src_re, src_im, dst, None)
        self._fn(self.state, ptr(src_re), ptr(src_im), ptr(dst))
        _check("transform")


class BatchPlan:
    """``batch`` dense transforms of one shape and kind (extension).

    ``form``: None / "plain" (FP32), "tc" (split-precision tensor cores) or
    "f64" (double arrays, FP64 arithmetic).  ``__call__`` is synchronous (like
    afft); ``launch`` enqueues on a CUDA stream (device pointers only) and
    returns immediately.
    """

    def __init__(self, kind, dims, batch, fmt=afft_split, form=None):
        L = lib()
        self.kind = KINDS[kind] if isinstance(kind, str) else kind
        self.dims = [int(d) for d in dims]
        self.batch = int(batch)
        self.format = fmt
        self.form = form
        if form == "tc":
            fmt = fmt | FORM_TC
        elif form == "f64":
            fmt = fmt | FORM_F64
        elif form not in (None, "plain"):
            raise ValueError("form must be None, 'plain', 'tc' or 'f64'")
        arr, n = _dims(self.dims)
        size = L.afft_gb300_batch_memsize(self.kind, n, arr, self.batch, fmt)
        self.state = None
        if size == 0 or size == ctypes.c_size_t(-1).value:
            _check("batch_memsize")
            raise AfftError("batch_memsize rejected the plan")
        self._mem = ctypes.create_string_buffer(size)
        self.state = L.afft_gb300_batch_create(self.kind, n, arr, self.batch, fmt, ctypes.addressof(self._mem))
        if not self.state:
            _check("batch_create")
            raise AfftError("batch_create failed")
        name = {KIND_C: "c", KIND_CI: "ci", KIND_R: "r", KIND_RI: "ri"}[self.kind]
        self._fn = getattr(L, "afft_%d_%s_transform" % (64 if form == "f64" else 32, name))

    def __call__(self, a, b=None, c=None, d=None):
        bits = 64 if self.form == "f64" else 32
        if self.kind in (KIND_C, KIND_CI):
            _validate(self.kind, self.dims, self.batch, self.format, bits, a, b, c, d)
            self._fn(self.state, ptr(a), ptr(b), ptr(c), ptr(d))
        elif self.kind == KIND_R:
            _validate(self.kind, self.dims, self.batch, self.format, bits, a, None, b, c)
            self._fn(self.state, ptr(a), ptr(b), ptr(c))
        else:
            _validate(self.kind, self.dims, self.batch, self.format, bits, a, b, c, None)
            self._fn(self.state, ptr(a), ptr(b), ptr(c))
        _check("transform")

    def launch(self, src_re, src_im, dst_re, dst_im, stream=None):
        """Enqueue without waiting; ``stream`` is a torch.cuda.Stream, a raw
        cudaStream_t int, or None for the CUDA default stream."""
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _validate(self.kind, self.dims, self.batch, self.format, 64 if self.form == "f64" else 32,
                  src_re, src_im, dst_re, dst_im)
        rc = lib().afft_gb300_transform_async(self.state, ptr(src_re), ptr(src_im), ptr(dst_re), ptr(dst_im), s)
        if rc:
            _check("transform_async")

    @property
    def launches(self):
        return lib().afft_gb300_plan_launches(self.state)

    def release(self):
        if self.state:
            lib().afft_gb300_release(self.state)
            self.state = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Queue:
    """Many transforms of mixed sizes and kinds run as one unit (extension).

    ``descs``: iterable of (kind, dims, src_re, src_im, dst_re, dst_im) with
    device arrays.
    """

    def __init__(self, descs, form=None, tuned=False):
        items = list(descs)
        arr = (Desc * max(1, len(items)))()
        for i, (kind, dims, sr, si, dr, di) in enumerate(items):
            d = arr[i]
            d.kind = KINDS[kind] if isinstance(kind, str) else kind
            d.ndim = len(dims)   # the library rejects ndim outside 1..3
            for j, x in enumerate(dims[:3]):
                d.dim[j] = int(x)
            d.src_re, d.src_im, d.dst_re, d.dst_im = ptr(sr), ptr(si), ptr(dr), ptr(di)
        flags = (FORM_TC if form == "tc" else 0) | (QUEUE_TUNED if tuned else 0)
        self._q = lib().afft_gb300_queue_create_ex(arr, len(items), flags)
        if not self._q:
            _check("queue_create")
            raise AfftError("queue_create failed")

    def run(self, stream=None):
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        if lib().afft_gb300_queue_run(self._q, s):
            _check("queue_run")

    @property
    def launches(self):
        return lib().afft_gb300_queue_launches(self._q)

    def __del__(self):
        q = getattr(self, "_q", None)
        if q:
            lib().afft_gb300_queue_destroy(q)
            self._q = None
