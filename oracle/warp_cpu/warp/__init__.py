"""A CPU stand-in for the parts of NVIDIA Warp's Python API that flub's
projection path uses -- TEST INFRASTRUCTURE ONLY.

It exists so that the reference's own kernel files (multigrid/mgpcg.py,
divergence.py, subtract_gradient.py, geometry.py, const_param.py,
utils/util.py of Luke-Skycrawler/flub) can be imported and executed
UNMODIFIED on the CPU to generate golden fixtures
(tests/golden/make_ref_golden.py).  Warp itself (the third-party package
``warp-lang``; the reference pins no version) cannot be installed here.
Nothing under flub_gb300/ may import this module.

Execution model (a restatement of Warp's documented semantics, not of its
code):

* ``@kernel`` functions run one thread at a time, in row-major order of the
  launch dimensions, with ``tid()`` returning the current thread's index.
  Race-free kernels give the same result in any order; the reference's one
  scatter with atomics (``_restrict_mcadams``) is thereby fixed to that
  sequential order.
* ``float`` in a kernel is FP32: arrays hold ``numpy.float32``, scalar kernel
  arguments annotated ``float`` are rounded to FP32 at launch, ``constant``
  turns Python floats into FP32, and vector components are FP32.  The bodies
  of ``@kernel`` and ``@func`` functions are recompiled from their source so
  that every float literal, and every module-level Python float they read, is
  an FP32 constant, as Warp's code generator makes them: ``2.0 / 9.0`` is an
  FP32 division at run time, not a double folded by Python.  Every arithmetic
  operation of the bodies is then an IEEE FP32 operation (numpy >= 2
  promotion rules keep Python ints and floats produced at run time, such as
  ``float(i)``, weak against FP32), evaluated without FMA contraction.  Host
  code of the reference modules is left as it is.
* ``empty`` returns zero-filled memory (Warp leaves it uninitialised).
* Between ``capture_begin`` and ``capture_end`` launches and array fills are
  recorded, not executed; ``capture_launch`` replays them.  This is what makes
  the reference's first ``graph_precondition`` call (multigrid/mgpcg.py:286-294)
  a no-op, as it is under Warp.

Builtins restated from Warp's published definitions (warp/native/vec.h,
quat.h, builtins): componentwise vector ``min``/``max`` and their one-argument
reductions, ``where``, ``clamp``, ``length`` = sqrt(dot), ``dot`` summed left to
right, ``cross``, ``quat_rotate_inv(q, x) = x (2w^2 - 1) - cross(q.xyz, x) w 2 +
q.xyz dot(q.xyz, x) 2``, ``atomic_add`` returning the old value.
"""
import ast
import builtins
import inspect
import math
import textwrap

import numpy as np

_f32 = np.float32

# ----------------------------------------------------------------- scalar types

float32 = np.float32
float64 = np.float64
int32 = np.int32
int64 = np.int64
uint64 = np.uint64
uint8 = np.uint8
int = builtins.int  # noqa: A001  (wp.int in annotations)
pi = _f32(math.pi)
inf = _f32(np.inf)


def constant(x):
    """wp.constant: a compile-time constant; Python floats become FP32."""
    if isinstance(x, builtins.bool):
        return x
    if isinstance(x, builtins.float):
        return _f32(x)
    return x


def _np_dtype(dtype):
    if dtype is builtins.float or dtype is np.float32:
        return np.float32
    if dtype is np.float64:
        return np.float64
    if dtype is builtins.int or dtype is np.int32:
        return np.int32
    if dtype is np.int64:
        return np.int64
    if dtype is np.uint8:
        return np.uint8
    if dtype is builtins.bool:
        return np.bool_
    return None  # vector / struct element types: object arrays


# ----------------------------------------------------------------- vectors

class _Vec:
    __slots__ = ("c",)
    N = 3
    FLOAT = True
    # numpy scalars defer to the vector's own operators (an FP32 scalar times
    # a vector is a vector, not an array built from its components)
    __array_ufunc__ = None

    def __init__(self, *args):
        if len(args) == 1 and isinstance(args[0], (_Vec, list, tuple, np.ndarray)):
            vals = list(args[0])
        elif len(args) == 0:
            vals = [0] * self.N
        elif len(args) == 1:
            vals = [args[0]] * self.N
        else:
            vals = list(args)
        if len(vals) != self.N:
            raise ValueError(f"{type(self).__name__} needs {self.N} components")
        self.c = [_f32(v) for v in vals] if self.FLOAT else [builtins.int(v) for v in vals]

    def _new(self, vals):
        v = object.__new__(type(self))
        v.c = vals
        return v

    def __getitem__(self, i):
        return self.c[i]

    def __setitem__(self, i, val):
        self.c[i] = _f32(val) if self.FLOAT else builtins.int(val)

    def __len__(self):
        return self.N

    def __iter__(self):
        return iter(self.c)

    def __add__(self, o):
        return self._new([a + b for a, b in zip(self.c, o.c)])

    def __sub__(self, o):
        return self._new([a - b for a, b in zip(self.c, o.c)])

    def __neg__(self):
        return self._new([-a for a in self.c])

    def __mul__(self, s):
        if isinstance(s, _Vec):
            raise TypeError("vector * vector: use dot/cross")
        return self._new([a * s for a in self.c])

    def __rmul__(self, s):
        return self._new([s * a for a in self.c])

    def __truediv__(self, s):
        return self._new([a / s for a in self.c])

    def __eq__(self, o):
        return isinstance(o, _Vec) and all(a == b for a, b in zip(self.c, o.c))

    def __ne__(self, o):
        return not self.__eq__(o)

    __hash__ = None

    def __repr__(self):
        return f"{type(self).__name__}({', '.join(str(a) for a in self.c)})"


class vec3(_Vec):
    __slots__ = ()
    N = 3


class vec4(_Vec):
    __slots__ = ()
    N = 4


class vec3i(_Vec):
    __slots__ = ()
    N = 3
    FLOAT = False


class quat(_Vec):
    """(x, y, z, w) storage, as Warp's quat."""
    __slots__ = ()
    N = 4

    def __mul__(self, o):
        if not isinstance(o, quat):
            return _Vec.__mul__(self, o)
        a, b = self.c, o.c
        return quat(a[3] * b[0] + b[3] * a[0] + a[1] * b[2] - a[2] * b[1],
                    a[3] * b[1] + b[3] * a[1] + a[2] * b[0] - a[0] * b[2],
                    a[3] * b[2] + b[3] * a[2] + a[0] * b[1] - a[1] * b[0],
                    a[3] * b[3] - (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]))


class transform:
    """wp.transform: a position and a rotation (the reference only names the
    type in kernel signatures and builds it from (p, q))."""

    def __init__(self, p=None, q=None):
        self.p = vec3(p) if p is not None else vec3()
        self.q = quat(q) if q is not None else quat(0.0, 0.0, 0.0, 1.0)


class spatial_vector(_Vec):
    """wp.spatial_vector: 6 FP32 components (angular, then linear)."""
    __slots__ = ()
    N = 6

    def __init__(self, *args):
        if len(args) == 2 and all(isinstance(a, _Vec) for a in args):
            args = (list(args[0]) + list(args[1]),)
        super().__init__(*args)


class types:
    """wp.types.vector(length, dtype): a fixed-length FP32 (or int) vector type."""

    @staticmethod
    def vector(length, dtype=builtins.float):
        return type(f"vec{length}", (_Vec,), {"__slots__": (), "N": builtins.int(length),
                                              "FLOAT": dtype is not builtins.int and dtype is not np.int32})


def quat_identity():
    return quat(0.0, 0.0, 0.0, 1.0)


def quat_inverse(q):
    return quat(-q[0], -q[1], -q[2], q[3])


def dot(a, b):
    s = a[0] * b[0]
    for i in range(1, len(a)):
        s = s + a[i] * b[i]
    return s


def cross(a, b):
    return vec3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def length(v):
    return np.sqrt(_f32(dot(v, v)))


def normalize(v):
    n = length(v)
    return v / n if n > 0 else vec3(0.0, 0.0, 0.0)


def quat_rotate_inv(q, x):
    w = q[3]
    qv = vec3(q[0], q[1], q[2])
    c = _f32(2.0) * w * w - _f32(1.0)
    return x * c - cross(qv, x) * w * _f32(2.0) + qv * dot(qv, x) * _f32(2.0)


def quat_rotate(q, x):
    w = q[3]
    qv = vec3(q[0], q[1], q[2])
    c = _f32(2.0) * w * w - _f32(1.0)
    return x * c + cross(qv, x) * w * _f32(2.0) + qv * dot(qv, x) * _f32(2.0)


# ----------------------------------------------------------------- scalar builtins

def where(cond, a, b):
    return a if cond else b


def min(a, b=None):  # noqa: A001
    if b is None:
        r = a[0]
        for x in a.c[1:]:
            if x < r:
                r = x
        return r
    if isinstance(a, _Vec):
        return a._new([x if x < y else y for x, y in zip(a.c, b.c)])
    return a if a < b else b


def max(a, b=None):  # noqa: A001
    if b is None:
        r = a[0]
        for x in a.c[1:]:
            if x > r:
                r = x
        return r
    if isinstance(a, _Vec):
        return a._new([x if x > y else y for x, y in zip(a.c, b.c)])
    return a if a > b else b


def clamp(x, lo, hi):
    return min(max(x, lo), hi)


def abs(x):  # noqa: A001
    if isinstance(x, _Vec):
        return x._new([builtins.abs(a) for a in x.c])
    return builtins.abs(x)


def sign(x):
    return _f32(-1.0) if x < 0 else _f32(1.0)


def floor(x):
    return np.floor(_f32(x))


def ceil(x):
    return np.ceil(_f32(x))


def sqrt(x):
    return np.sqrt(_f32(x))


def cos(x):
    return np.cos(_f32(x))


def sin(x):
    return np.sin(_f32(x))


def exp(x):
    return np.exp(_f32(x))


def lerp(a, b, t):
    return a * (_f32(1.0) - t) + b * t


# ----------------------------------------------------------------- arrays

class _Annot:
    """What wp.array3d(dtype=...) evaluates to in an annotation."""

    def __init__(self, dtype, ndim):
        self.dtype, self.ndim = dtype, ndim


class _NumArray(np.ndarray):
    """A Warp array of a scalar type: a numpy array with Warp's methods."""

    def numpy(self):
        return np.asarray(self)

    def zero_(self):
        _enqueue(lambda: np.ndarray.fill(self, 0))

    def fill_(self, value):
        _enqueue(lambda: np.ndarray.fill(self, value))

    def assign(self, src):
        np.copyto(np.asarray(self), np.asarray(src))


class _ObjArray:
    """A Warp array of vectors or structs (1-D), e.g. positions, quaternions,
    geometry descriptors."""

    def __init__(self, items):
        self.items = list(items)
        self.shape = (len(self.items),)

    def __getitem__(self, i):
        return self.items[i]

    def __setitem__(self, i, v):
        self.items[i] = v

    def __len__(self):
        return len(self.items)

    def numpy(self):
        return np.array([list(v) if isinstance(v, _Vec) else v for v in self.items])


def _shape(shape):
    if isinstance(shape, (tuple, list)):
        return tuple(builtins.int(s) for s in shape)
    return (builtins.int(shape),)


def _make(shape, dtype, fill):
    nd = _np_dtype(dtype)
    if nd is None:
        assert len(_shape(shape)) == 1, "vector/struct arrays are 1-D here"
        return _ObjArray([dtype() for _ in range(_shape(shape)[0])])
    a = np.full(_shape(shape), fill, dtype=nd).view(_NumArray)
    return a


def zeros(shape, dtype=builtins.float, device=None, **kw):
    return _make(shape, dtype, 0)


def empty(shape, dtype=builtins.float, device=None, **kw):
    return _make(shape, dtype, 0)


def zeros_like(a):
    return np.zeros_like(np.asarray(a)).view(_NumArray)


def empty_like(a):
    return zeros_like(a)


def array(data=None, dtype=builtins.float, shape=None, ndim=None, device=None, **kw):
    if data is None:
        return _Annot(dtype, ndim)
    nd = _np_dtype(dtype)
    if nd is None:
        return _ObjArray([d if isinstance(d, (_Vec,)) or not hasattr(dtype, "N") else dtype(d) for d in data])
    a = np.array(data, dtype=nd)
    if shape is not None:
        a = a.reshape(_shape(shape))
    return a.view(_NumArray)


def from_numpy(arr, dtype=builtins.float, shape=None, device=None, **kw):
    return array(arr, dtype=dtype, shape=shape)


def array1d(dtype=builtins.float, **kw):
    return _Annot(dtype, 1)


def array2d(dtype=builtins.float, **kw):
    return _Annot(dtype, 2)


def array3d(dtype=builtins.float, **kw):
    return _Annot(dtype, 3)


def copy(dest, src, dest_offset=0, src_offset=0, count=0):
    _enqueue(lambda: np.copyto(np.asarray(dest), np.asarray(src)))


# ----------------------------------------------------------------- structs

def struct(cls):
    """@wp.struct: a plain attribute holder with the annotated fields."""
    fields = dict(getattr(cls, "__annotations__", {}))

    def __init__(self):
        for name in fields:
            setattr(self, name, None)

    cls.__init__ = __init__
    cls._wp_fields = fields
    return cls


# ----------------------------------------------------------------- kernels, launches, capture

_tid = None
_capture = None


def tid():
    return _tid


def _enqueue(fn):
    if _capture is not None:
        _capture.append(fn)
    else:
        fn()


def _wp_f32(x):
    return _f32(x)


def _wp_glob(x):
    """A module-level name read by kernel code: Python floats are FP32
    constants there (bool is left alone)."""
    return _f32(x) if type(x) is builtins.float else x


class _Fp32Source(ast.NodeTransformer):
    """Float literals -> _wp_f32(literal); reads of names that are not local
    to the function -> _wp_glob(name)."""

    def __init__(self, local_names):
        self.local_names = local_names

    def visit_Constant(self, node):
        if type(node.value) is builtins.float:
            return ast.copy_location(ast.Call(ast.Name("_wp_f32", ast.Load()), [node], []), node)
        return node

    def visit_Name(self, node):
        if isinstance(node.ctx, ast.Load) and node.id not in self.local_names:
            return ast.copy_location(ast.Call(ast.Name("_wp_glob", ast.Load()), [node], []), node)
        return node


def _fp32_function(f):
    """f recompiled from its source with _Fp32Source, in f's own module
    namespace (which gains the two helper names)."""
    src = textwrap.dedent(inspect.getsource(f))
    tree = ast.parse(src)
    ast.increment_lineno(tree, f.__code__.co_firstlineno - 1)  # tracebacks point into the reference file
    fn = tree.body[0]
    fn.decorator_list = []
    local_names = {a.arg for a in fn.args.args + fn.args.kwonlyargs + fn.args.posonlyargs}
    if fn.args.vararg:
        local_names.add(fn.args.vararg.arg)
    if fn.args.kwarg:
        local_names.add(fn.args.kwarg.arg)
    for node in ast.walk(fn):
        if isinstance(node, ast.Name) and isinstance(node.ctx, (ast.Store, ast.Del)):
            local_names.add(node.id)
    # defaults and annotations are evaluated at definition time: leave them
    new_body = [_Fp32Source(local_names).visit(b) for b in fn.body]
    fn.body = new_body
    ast.fix_missing_locations(tree)
    g = f.__globals__
    g.setdefault("_wp_f32", _wp_f32)
    g.setdefault("_wp_glob", _wp_glob)
    ns = {}
    exec(compile(tree, inspect.getsourcefile(f) or "<kernel>", "exec"), g, ns)
    out = ns[f.__name__]
    out.__wrapped__ = f
    return out


def func(f):
    return _fp32_function(f)


class Kernel:
    def __init__(self, f):
        self.func = _fp32_function(f)
        self.__name__ = f.__name__
        self.key = f.__name__
        sig = inspect.signature(f)
        self.casts = []
        for name, p in sig.parameters.items():
            a = p.annotation
            if a is builtins.float or a is np.float32:
                self.casts.append(_f32)
            elif a is builtins.int or a is np.int32:
                self.casts.append(builtins.int)
            elif isinstance(a, type) and issubclass(a, _Vec):
                self.casts.append(a)
            else:
                self.casts.append(None)

    def __call__(self, *args):
        raise RuntimeError("Warp kernels are launched with wp.launch")


def kernel(f=None, **kw):
    if f is None:
        return lambda g: Kernel(g)
    return Kernel(f)


def _run(k, dim, args):
    global _tid
    f = k.func
    dims = _shape(dim)
    try:
        if len(dims) == 1:
            for i in range(dims[0]):
                _tid = i
                f(*args)
        elif len(dims) == 2:
            for i in range(dims[0]):
                for j in range(dims[1]):
                    _tid = (i, j)
                    f(*args)
        elif len(dims) == 3:
            for i in range(dims[0]):
                for j in range(dims[1]):
                    for kk in range(dims[2]):
                        _tid = (i, j, kk)
                        f(*args)
        else:
            for idx in np.ndindex(*dims):
                _tid = tuple(builtins.int(x) for x in idx)
                f(*args)
    finally:
        _tid = None


def _cast(c, a):
    """Scalar kernel arguments take the parameter's type (a Python float
    passed for a ``float`` parameter becomes FP32, as Warp converts it)."""
    if c is None or isinstance(a, c if isinstance(c, type) else ()):
        return a
    return c(a)


def launch(kernel, dim, inputs=(), outputs=(), device=None, stream=None, **kw):
    args = list(inputs) + list(outputs)
    if len(args) != len(kernel.casts):
        raise TypeError(f"{kernel.key}: {len(args)} arguments for {len(kernel.casts)} parameters")
    args = [_cast(c, a) for c, a in zip(kernel.casts, args)]
    _enqueue(lambda: _run(kernel, dim, args))


class Graph:
    def __init__(self, ops):
        self.ops = ops


def capture_begin(device=None, stream=None, **kw):
    global _capture
    if _capture is not None:
        raise RuntimeError("capture already active")
    _capture = []


def capture_end(device=None, stream=None, **kw):
    global _capture
    ops, _capture = _capture, None
    return Graph(ops)


def capture_launch(graph, stream=None):
    for op in graph.ops:
        op()


# ----------------------------------------------------------------- atomics

def atomic_add(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx)
    old = arr[idx]
    arr[idx] = old + value
    return old


def atomic_sub(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx)
    old = arr[idx]
    arr[idx] = old - value
    return old


def atomic_min(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx)
    old = arr[idx]
    arr[idx] = min(old, value)
    return old


def atomic_max(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx)
    old = arr[idx]
    arr[idx] = max(old, value)
    return old


# ----------------------------------------------------------------- runtime odds and ends

def init():
    pass


def synchronize():
    pass


class ScopedTimer:
    def __init__(self, name="", active=True, synchronize=False, **kw):
        self.name = name

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


class config:
    mode = "release"
    verify_fp = False
