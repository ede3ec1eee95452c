"""TEST INFRASTRUCTURE ONLY: ctypes front end of the CPU oracle (liboracle.so).

Loaded by tests/, the smoke check and bench.py's CPU-baseline leg, and by
nothing in the product package.  Two restatements of afft's power-of-two FFT
path live behind it (see afft_oracle.h for file:line citations):

* ``c2c64`` / ``r2c64`` / ``c2r64`` -- the FP64 oracle of the reference test
  harness (testing.cpp:870-1002), radix-2 Stockham with directly computed
  twiddles; the numerical ground truth.
* ``Port32`` -- a scalar FP32 port of afft's own algorithm (radix-4 passes,
  recurrence twiddles, real pre/post pass), the CPU baseline ("port").

Also ``ref_lib()``: the reference library itself, when oracle/_ref was built
here from the reference's sources (x86-64 only); used to pin the oracle and to
generate the golden fixtures.  ``RefBatch`` / ``ref_mixed`` drive the
reference library (every backend on x86-64, or its scalar backend built on
any host from the staged sources) through its own C API over many
transforms and host threads: the CPU baseline when it is available.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libafft_ref.so")
REF_SCALAR_PATH = os.path.join(HERE, "_ref", "libafft_ref_scalar.so")

C, CI, R, RI = 0, 1, 2, 3
KINDS = {"c": C, "ci": CI, "r": R, "ri": RI}

_lib = None


def build():
    """Compile liboracle.so with make (gcc only, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        L.oracle_mt19937_uniform.argtypes = [ctypes.c_uint32, I64, ctypes.c_float, ctypes.c_float, P]
        L.oracle_mt19937_uniform.restype = None
        L.oracle_mt19937_raw.argtypes = [ctypes.c_uint32, I64, P]
        L.oracle_mt19937_raw.restype = None
        for name in ("oracle64_c2c",):
            getattr(L, name).argtypes = [ctypes.c_int, P, ctypes.c_int, P, P, P, P]
        L.oracle64_r2c.argtypes = [ctypes.c_int, P, P, P, P]
        L.oracle64_c2r.argtypes = [ctypes.c_int, P, P, P, P]
        for pre in ("port32", "port64"):
            getattr(L, pre + "_plan_create").argtypes = [ctypes.c_int, ctypes.c_int, P]
            getattr(L, pre + "_plan_create").restype = P
            getattr(L, pre + "_plan_destroy").argtypes = [P]
            getattr(L, pre + "_plan_in_elems").argtypes = [P]
            getattr(L, pre + "_plan_in_elems").restype = I64
            getattr(L, pre + "_plan_out_elems").argtypes = [P]
            getattr(L, pre + "_plan_out_elems").restype = I64
            getattr(L, pre + "_execute").argtypes = [P, P, P, P, P]
            getattr(L, pre + "_execute_batch").argtypes = [P, I64, ctypes.c_int, P, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _dims(dims):
    return np.ascontiguousarray(np.array(dims, dtype=np.int64))


def squeeze(dims):
    """common.hpp:68-84: drop size-1 dims (keep one if all are 1)."""
    d = [int(x) for x in dims if int(x) != 1]
    return d or [1]


def half_elems(dims):
    """Elements per array of a real transform's half spectrum: dim 0 halved."""
    d = squeeze(dims)
    return (d[0] // 2 + 1) * int(np.prod(d[1:], dtype=np.int64))


def mt19937_uniform(count, seed=5489, lo=-1.0, hi=1.0):
    """The reference harness input generator (testing.cpp:1064-1067);
    std::mt19937's default seed is 5489."""
    out = np.empty(count, np.float32)
    lib().oracle_mt19937_uniform(seed, count, lo, hi, _p(out))
    return out


def mt19937_raw(count, seed=5489):
    out = np.empty(count, np.uint32)
    lib().oracle_mt19937_raw(seed, count, _p(out))
    return out


def c2c64(dims, re, im, inverse=False):
    re = np.ascontiguousarray(re, np.float64).ravel()
    im = np.ascontiguousarray(im, np.float64).ravel()
    ore = np.empty_like(re)
    oim = np.empty_like(im)
    d = _dims(dims)
    rc = lib().oracle64_c2c(len(d), _p(d), int(inverse), _p(re), _p(im), _p(ore), _p(oim))
    if rc:
        raise ValueError("invalid shape %r" % (dims,))
    return ore, oim


def r2c64(dims, x):
    x = np.ascontiguousarray(x, np.float64).ravel()
    h = half_elems(dims)
    ore = np.empty(h)
    oim = np.empty(h)
    d = _dims(dims)
    if lib().oracle64_r2c(len(d), _p(d), _p(x), _p(ore), _p(oim)):
        raise ValueError("invalid shape %r" % (dims,))
    return ore, oim


def c2r64(dims, re, im):
    re = np.ascontiguousarray(re, np.float64).ravel()
    im = np.ascontiguousarray(im, np.float64).ravel()
    out = np.empty(int(np.prod(dims, dtype=np.int64)))
    d = _dims(dims)
    if lib().oracle64_c2r(len(d), _p(d), _p(re), _p(im), _p(out)):
        raise ValueError("invalid shape %r" % (dims,))
    return out


def oracle64(kind, dims, a, b=None):
    """Dispatch by afft kind name ('c', 'ci', 'r', 'ri'); returns float64
    arrays: (re, im) for c/ci/r, the real array for ri."""
    if kind == "c":
        return c2c64(dims, a, b, False)
    if kind == "ci":
        return c2c64(dims, a, b, True)
    if kind == "r":
        return r2c64(dims, a)
    if kind == "ri":
        return c2r64(dims, a, b)
    raise ValueError(kind)


class Port32:
    """FP32 port of afft (CPU baseline).  Dense batches of one shape."""

    PREFIX = "port32"
    DTYPE = np.float32

    def __init__(self, kind, dims):
        self.kind = kind
        self.dims = list(dims)
        d = _dims(dims)
        self._fn = lambda name: getattr(lib(), self.PREFIX + "_" + name)
        self._h = self._fn("plan_create")(KINDS[kind], len(d), _p(d))
        if not self._h:
            raise ValueError("invalid shape %r" % (dims,))
        self.in_elems = self._fn("plan_in_elems")(self._h)
        self.out_elems = self._fn("plan_out_elems")(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._fn("plan_destroy")(h)
            self._h = None

    def __call__(self, a, b=None, batch=1, threads=1, out=None):
        a = np.ascontiguousarray(a, self.DTYPE).ravel()
        b = None if b is None else np.ascontiguousarray(b, self.DTYPE).ravel()
        if out is None:
            ore = np.empty(batch * self.out_elems, self.DTYPE)
            oim = None if self.kind == "ri" else np.empty(batch * self.out_elems, self.DTYPE)
        else:
            ore, oim = out
        rc = self._fn("execute_batch")(self._h, batch, threads, _p(a), _p(b), _p(ore), _p(oim))
        if rc:
            raise RuntimeError(self.PREFIX + " failed")
        return ore if self.kind == "ri" else (ore, oim)


class Port64(Port32):
    """FP64 port of afft (the CPU baseline of the afft_64_* path)."""

    PREFIX = "port64"
    DTYPE = np.float64


_ref = None


def ref_available():
    return os.path.exists(REF_PATH)


def ref_lib():
    """The reference afft library built from its own sources (x86-64 here)."""
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_PATH)
        P = ctypes.c_void_p
        S = ctypes.c_size_t
        for bits in ("32", "64"):
            for k in ("c", "ci", "r", "ri"):
                ms = getattr(L, "afft_%s_%s_memsize" % (bits, k))
                ms.restype = S
                ms.argtypes = [S, P, ctypes.c_int, ctypes.c_int]
                cr = getattr(L, "afft_%s_%s_create" % (bits, k))
                cr.restype = P
                cr.argtypes = [S, P, ctypes.c_int, P, ctypes.c_int]
                tr = getattr(L, "afft_%s_%s_transform" % (bits, k))
                tr.restype = None
                tr.argtypes = [P, P, P, P, P] if k in ("c", "ci") else [P, P, P, P]
        L.afft_supported.argtypes = [ctypes.c_int]
        _ref = L
    return _ref


def ref_run(kind, dims, a, b=None, impl=0, bits=32):
    """One transform through the reference library's own C API (fft.h):
    afft_32_* on float arrays, or afft_64_* on double arrays (bits=64)."""
    L = ref_lib()
    dt = np.float32 if bits == 32 else np.float64
    fn = lambda what: getattr(L, "afft_%d_%s_%s" % (bits, kind, what))
    d = np.array(dims, dtype=np.uint64)
    ms = fn("memsize")(len(d), _p(d), 0, impl)
    if ms == 0:
        raise ValueError("reference rejected %r impl=%d" % (dims, impl))
    mem = np.zeros(ms + 64, np.uint8)
    st = fn("create")(len(d), _p(d), 0, _p(mem), impl)
    n = int(np.prod(dims, dtype=np.int64))
    h = half_elems(dims)
    a = np.ascontiguousarray(a, dt).ravel()
    b = None if b is None else np.ascontiguousarray(b, dt).ravel()
    if kind in ("c", "ci"):
        ore = np.zeros(n, dt)
        oim = np.zeros(n, dt)
        fn("transform")(ctypes.c_void_p(st), _p(a), _p(b), _p(ore), _p(oim))
        return ore, oim
    if kind == "r":
        ore = np.zeros(h, dt)
        oim = np.zeros(h, dt)
        fn("transform")(ctypes.c_void_p(st), _p(a), _p(ore), _p(oim))
        return ore, oim
    out = np.zeros(n, dt)
    fn("transform")(ctypes.c_void_p(st), _p(a), _p(b), _p(out))
    return out


def rel_l2(y, ref):
    """Standard relative L2 error ||y - ref|| / ||ref|| over all arrays."""
    ys = y if isinstance(y, (tuple, list)) else (y,)
    rs = ref if isinstance(ref, (tuple, list)) else (ref,)
    num = sum(float(np.sum((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)) for a, b in zip(ys, rs))
    den = sum(float(np.sum(np.asarray(b, np.float64) ** 2)) for b in rs)
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


def max_rel(y, ref):
    """max |y - ref| / max |ref| over all arrays."""
    ys = y if isinstance(y, (tuple, list)) else (y,)
    rs = ref if isinstance(ref, (tuple, list)) else (ref,)
    num = max(float(np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)))) for a, b in zip(ys, rs))
    den = max(float(np.max(np.abs(np.asarray(b, np.float64)))) for b in rs)
    return num / den if den > 0 else num


def afft_error(y, ref):
    """The reference harness metric (testing.cpp:1113-1129):
    sqrt(sum (y-ref)^2 / sum (y^2 + ref^2))."""
    ys = y if isinstance(y, (tuple, list)) else (y,)
    rs = ref if isinstance(ref, (tuple, list)) else (ref,)
    num = sum(float(np.sum((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)) for a, b in zip(ys, rs))
    den = sum(float(np.sum(np.asarray(a, np.float64) ** 2 + np.asarray(b, np.float64) ** 2)) for a, b in zip(ys, rs))
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


_bench = {}


def ref_bench_lib():
    """(library, impl id, description) of the reference afft build that the
    CPU baseline times, or None: every backend with afft_auto picking the
    best (x86-64), else the scalar backend, the one afft builds on Arm."""
    for path, impl, what in ((REF_PATH, 0, "afft, best SIMD backend (afft_auto)"),
                             (REF_SCALAR_PATH, 1, "afft, scalar backend (the backend afft builds on this host)")):
        if path in _bench:
            if _bench[path] is not None:
                return _bench[path]
            continue
        got = None
        if os.path.exists(path):
            try:
                L = ctypes.CDLL(path)
                P, I64 = ctypes.c_void_p, ctypes.c_int64
                L.refbatch_ctx_create.restype = P
                L.refbatch_ctx_create.argtypes = [ctypes.c_int]
                L.refbatch_ctx_destroy.argtypes = [P]
                L.refbatch_uniform.restype = ctypes.c_int
                L.refbatch_uniform.argtypes = [P, ctypes.c_int, ctypes.c_size_t, P, I64, ctypes.c_int, ctypes.c_int,
                                               P, P, P, P]
                L.refbatch_mixed.restype = ctypes.c_int
                L.refbatch_mixed.argtypes = [P, I64, P, P, P, P, P, P, P, ctypes.c_int, ctypes.c_int]
                got = (L, impl, what)
            except (OSError, AttributeError):
                got = None
        _bench[path] = got
        if got is not None:
            return got
    return None


class RefBatch:
    """Dense batches of one shape through the reference afft library's C
    API, split over host threads with one plan per thread (afft plans are
    not reentrant).  Same call form as Port32."""

    DTYPE = np.float32

    def __init__(self, kind, dims, threads):
        got = ref_bench_lib()
        if got is None:
            raise RuntimeError("reference afft library not built")
        self.L, self.impl, self.what = got
        self.kind = kind
        self.dims = squeeze(dims)
        self.threads = max(1, int(threads))
        self._d = np.array(self.dims, dtype=np.uint64)
        n = int(np.prod(self.dims, dtype=np.int64))
        h = half_elems(self.dims)
        self.in_elems = h if kind == "ri" else n
        self.out_elems = h if kind == "r" else n
        self._ctx = self.L.refbatch_ctx_create(self.threads)
        if not self._ctx:
            raise MemoryError("refbatch context")

    def __del__(self):
        c = getattr(self, "_ctx", None)
        if c:
            self.L.refbatch_ctx_destroy(c)
            self._ctx = None

    def __call__(self, a, b=None, batch=1, threads=None, out=None):
        a = np.ascontiguousarray(a, self.DTYPE).ravel()
        b = None if b is None else np.ascontiguousarray(b, self.DTYPE).ravel()
        if out is None:
            ore = np.empty(batch * self.out_elems, self.DTYPE)
            oim = None if self.kind == "ri" else np.empty(batch * self.out_elems, self.DTYPE)
        else:
            ore, oim = out
        t = min(self.threads, threads or self.threads)
        rc = self.L.refbatch_uniform(self._ctx, KINDS[self.kind], len(self._d), _p(self._d), batch, t, self.impl,
                                     _p(a), _p(b), _p(ore), _p(oim))
        if rc:
            raise RuntimeError("reference afft batch failed")
        return ore if self.kind == "ri" else (ore, oim)


class RefMixed:
    """Transforms of mixed shapes, each with its own arrays, through the
    reference afft library's C API: host threads take them from a shared
    counter, each keeping its own plans."""

    def __init__(self, threads):
        got = ref_bench_lib()
        if got is None:
            raise RuntimeError("reference afft library not built")
        self.L, self.impl, self.what = got
        self.threads = max(1, int(threads))
        self._ctx = self.L.refbatch_ctx_create(self.threads)
        self._keep = None

    def __del__(self):
        c = getattr(self, "_ctx", None)
        if c:
            self.L.refbatch_ctx_destroy(c)
            self._ctx = None

    def prepare(self, work):
        """work: list of (kind, dims, a, b, out_a, out_b) with numpy float32
        arrays (b / out_b None where the kind has none)."""
        m = len(work)
        kinds = np.array([KINDS[w[0]] for w in work], dtype=np.int32)
        ndims = np.array([len(squeeze(w[1])) for w in work], dtype=np.int32)
        dims = np.zeros((m, 3), dtype=np.uint64)
        for i, w in enumerate(work):
            d = squeeze(w[1])
            dims[i, :len(d)] = d
        ptr = lambda k: np.array([0 if w[k] is None else w[k].ctypes.data for w in work], dtype=np.uintp)
        self._keep = (work, kinds, ndims, dims, ptr(2), ptr(3), ptr(4), ptr(5))
        return m

    def run(self):
        work, kinds, ndims, dims, ia, ib, oa, ob = self._keep
        rc = self.L.refbatch_mixed(self._ctx, len(work), _p(kinds), _p(ndims), _p(dims), _p(ia), _p(ib), _p(oa),
                                   _p(ob), self.threads, self.impl)
        if rc:
            raise RuntimeError("reference afft mixed batch failed")
