"""Stand-in for numba (and cupy) under which the reference's numba-engine functions run as plain
Python in a container without numba, so that make_golden.py can record their outputs as fixtures.
Test infrastructure only: nothing in the package, the tests or the benchmark imports it.

What it reproduces:
  - @cuda.jit kernels run over the launch's threads, block after block, with cuda.grid(1)
    returning the thread's index; device functions are plain calls; cuda.local.array allocates a
    numpy array; device arrays are numpy arrays with copy_to_host; cuda.atomic.add / min update in
    place.  A kernel that calls cuda.syncthreads() runs its block's threads in lockstep from one
    barrier to the next (the call is rewritten as a yield), so what a thread reads after the
    barrier is what every thread of its block wrote before it.  Blocks run in launch order, so a
    value shared across blocks (the time kernel's wake time) is what the blocks before had
    written: a device may order its blocks otherwise, so fixtures that depend on it use one block.
  - numba's typing of constants.  numba types a float literal or a float global as float64 and an
    integer literal as int64, so `F = 1.0 / A` promotes a float32 determinant to FP64 and
    `-EPSILON < A` compares in FP64.  numpy keeps a float32 result when a Python scalar meets a
    float32 value, so the functions handed to cuda.jit are recompiled from their source text with
    every float / int / complex literal (and math.pi, cmath.pi, ...) wrapped as an np.float64 /
    np.int64 / np.complex128 value, and the modules' float globals are turned into np.float64
    (`freeze_float_globals`).  float32 x float32 stays float32, as in numba.
  - Structured arrays handed to a kernel are viewed as record arrays, whose elements give the
    attribute access of numba records (ray.dx) and write through to the array.
  - @njit / @jit / @guvectorize / @vectorize / prange run as plain Python and numpy.  The
    reference's njit code on the numba path (calc_dv_norm) computes in float32 under both: numba's
    ufunc typing keeps float32 ** int in float32, and nothing is fused without fastmath.
What it cannot reproduce: whether numba's NVVM build of a kernel fuses float32 products and sums
into FMAs.  Nothing is fused here, so decisions of the ray-triangle test can differ from a fused
build for pairs within rounding of a triangle edge.
"""
import ast
import inspect
import sys
import textwrap
import types

import numpy as np

_TID = [0]
_F64 = "_nbsim_f64"
_I64 = "_nbsim_i64"
_C128 = "_nbsim_c128"


class _Type:
    """A numba scalar type: indexable (float32[:, :]) and callable (float32(float32)) in signatures."""

    def __init__(self, name, dtype):
        self.name = name
        self.dtype = np.dtype(dtype) if dtype is not None else None

    def __getitem__(self, item):
        return self

    def __call__(self, *args):
        if args and not isinstance(args[0], _Type) and self.dtype is not None:
            return self.dtype.type(args[0])
        return self

    def __repr__(self):
        return f"numba_sim.{self.name}"


class _Record:
    """from_dtype(): usable as a numpy dtype (through .dtype) with numba's .size."""

    def __init__(self, dtype):
        self.dtype = np.dtype(dtype)
        self.size = self.dtype.itemsize


def _as_dtype(d):
    if isinstance(d, (_Type, _Record)):
        return d.dtype
    return np.dtype(d)


class _Literals(ast.NodeTransformer):
    """Wraps numeric literals (and math/cmath/np constants) in numba's literal types and turns
    statement-level cuda.syncthreads() calls into yields (block barriers)."""

    def visit_Expr(self, node):
        c = node.value
        if (isinstance(c, ast.Call) and isinstance(c.func, ast.Attribute) and c.func.attr == "syncthreads"):
            return ast.copy_location(ast.Expr(value=ast.Yield(value=None)), node)
        self.generic_visit(node)
        return node

    def visit_Constant(self, node):
        v = node.value
        if type(v) is float:
            fn = _F64
        elif type(v) is int:
            fn = _I64
        elif type(v) is complex:
            fn = _C128
        else:
            return node
        return ast.copy_location(ast.Call(func=ast.Name(id=fn, ctx=ast.Load()), args=[node], keywords=[]), node)

    def visit_Attribute(self, node):
        self.generic_visit(node)
        if (isinstance(node.value, ast.Name) and node.value.id in ("math", "cmath", "np", "numpy")
                and node.attr in ("pi", "e", "tau", "inf", "nan")):
            return ast.copy_location(ast.Call(func=ast.Name(id=_F64, ctx=ast.Load()), args=[node], keywords=[]),
                                     node)
        return node


def _numba_typed(fn):
    """fn recompiled from its source with numba's literal types, resolving names in its module."""
    src = textwrap.dedent(inspect.getsource(fn))
    tree = ast.parse(src)
    fdef = tree.body[0]
    assert isinstance(fdef, ast.FunctionDef), fn
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_Literals().visit(tree))
    g = fn.__globals__
    g.setdefault(_F64, np.float64)
    g.setdefault(_I64, np.int64)
    g.setdefault(_C128, np.complex128)
    ns = {}
    exec(compile(tree, inspect.getsourcefile(fn) or "<numba_sim>", "exec"), g, ns)
    return ns[fdef.name]


def _kernel_arg(a):
    if isinstance(a, np.ndarray) and a.dtype.names is not None:
        return a.view(np.recarray)
    return a


class _Kernel:
    def __init__(self, fn):
        self.py = _numba_typed(fn)
        self.lockstep = inspect.isgeneratorfunction(self.py)
        self.__name__ = fn.__name__

    def __getitem__(self, cfg):
        nblocks, nthreads = int(np.prod(cfg[0])), int(np.prod(cfg[1]))

        def launch(*args):
            args = [_kernel_arg(a) for a in args]
            for b in range(nblocks):
                tids = range(b * nthreads, (b + 1) * nthreads)
                if not self.lockstep:
                    for t in tids:
                        _TID[0] = t
                        self.py(*args)
                    continue
                live = [(t, self.py(*args)) for t in tids]
                while live:  # every thread of the block runs to its next barrier (or its end)
                    nxt = []
                    for t, g in live:
                        _TID[0] = t
                        try:
                            next(g)
                            nxt.append((t, g))
                        except StopIteration:
                            pass
                    live = nxt
        return launch


class DeviceArray(np.ndarray):
    def copy_to_host(self, ary=None, stream=0):
        out = np.array(self).view(np.ndarray)
        if ary is not None:
            ary[...] = out
            return ary
        return out

    def get(self):
        return self.copy_to_host()


def _device(a):
    return np.array(a).view(DeviceArray)


def _cuda_jit(*args, **kw):
    if args and callable(args[0]) and not isinstance(args[0], _Type):
        return _Kernel(args[0])
    device = kw.get("device", False)

    def deco(fn):
        return _numba_typed(fn) if device else _Kernel(fn)
    return deco


def _passthrough(*args, **kw):
    if args and callable(args[0]) and not isinstance(args[0], (_Type, list, str)):
        return args[0]
    return lambda fn: fn


class _Context:
    class memory_manager:
        class deallocations:
            @staticmethod
            def clear():
                pass

    @staticmethod
    def get_memory_info():
        return 64 << 30, 96 << 30


def _to_device(a, stream=0, copy=True, to=None):
    if to is not None:
        to[...] = a
        return to
    return _device(a)


def _make_cuda():
    cuda = types.ModuleType("numba.cuda")
    cuda.jit = _cuda_jit
    cuda.grid = lambda ndim=1: _TID[0]
    cuda.syncthreads = lambda: None
    cuda.local = types.SimpleNamespace(array=lambda shape, dtype: np.zeros(shape, _as_dtype(dtype)))
    cuda.atomic = types.SimpleNamespace(add=_atomic_add, min=_atomic_min)
    cuda.to_device = _to_device
    cuda.device_array = lambda shape, dtype=np.float64, **kw: np.zeros(shape, _as_dtype(dtype)).view(DeviceArray)
    cuda.current_context = lambda: _Context
    cuda.select_device = lambda i: None
    cuda.close = lambda: None
    cuda.profile_start = cuda.profile_stop = lambda: None
    return cuda


def _index(idx):
    # numba lowers a float index of an atomic (the time kernel's floor-divided sample index) to an integer
    if isinstance(idx, (float, np.floating)):
        assert float(idx).is_integer(), idx
        return int(idx)
    return idx


def _atomic_add(arr, idx, val):
    idx = _index(idx)
    old = arr[idx]
    arr[idx] = old + val
    return old


def _atomic_min(arr, idx, val):
    idx = _index(idx)
    old = arr[idx]
    if val < old:
        arr[idx] = val
    return old


def _make_meshio():
    """meshio's Mesh and CellBlock as plain containers (the reference's model code takes meshes by
    isinstance and reads .points, .cells[i].type / .data and .point_data)."""
    m = types.ModuleType("meshio")

    class CellBlock:
        def __init__(self, cell_type, data):
            self.type = cell_type
            self.data = np.asarray(data)

    class Mesh:
        def __init__(self, points, cells, point_data=None, cell_data=None):
            self.points = np.asarray(points)
            self.cells = [c if isinstance(c, CellBlock) else CellBlock(c[0], c[1]) for c in cells]
            self.point_data = dict(point_data or {})
            self.cell_data = dict(cell_data or {})

    m.Mesh, m.CellBlock = Mesh, CellBlock
    return m


class _StubFinder:
    """Import hook giving an empty package for every module under `roots` (plotting and meshing
    libraries the reference imports at module level but the numba path never calls)."""

    def __init__(self, roots):
        self.roots = roots

    def find_spec(self, name, path=None, target=None):
        import importlib.machinery
        if name.split(".")[0] not in self.roots:
            return None
        return importlib.machinery.ModuleSpec(name, self, is_package=True)

    def create_module(self, spec):
        m = types.ModuleType(spec.name)
        m.__path__ = []
        m.__getattr__ = _stub_attr
        return m

    def exec_module(self, module):
        pass


def _stub_attr(attr):
    if attr.startswith("__"):
        raise AttributeError(attr)
    return types.SimpleNamespace()


def install():
    """Puts the stand-in modules into sys.modules (numba, numba.cuda, cupy and the reference's
    geometry / plotting imports that the numba path does not use)."""
    nb = types.ModuleType("numba")
    cuda = _make_cuda()
    nb.cuda = cuda
    for name, dt in (("float32", np.float32), ("float64", np.float64), ("complex64", np.complex64),
                     ("complex128", np.complex128), ("int32", np.int32), ("int64", np.int64),
                     ("boolean", np.bool_), ("uint8", np.uint8)):
        setattr(nb, name, _Type(name, dt))
    nb.jit = nb.njit = nb.guvectorize = nb.vectorize = _passthrough
    nb.prange = range
    nb.from_dtype = _Record
    sys.modules["numba"] = nb
    sys.modules["numba.cuda"] = cuda
    cp = types.ModuleType("cupy")
    cp.zeros = lambda shape, dtype=np.float64: np.zeros(shape, dtype).view(DeviceArray)
    cp.asnumpy = lambda a: np.array(a).view(np.ndarray)
    cp.asarray = _device
    sys.modules["cupy"] = cp
    sys.modules["meshio"] = _make_meshio()
    sys.meta_path.insert(0, _StubFinder(("gmsh", "pyvista", "matplotlib", "mpl_toolkits", "pylab",
                                         "importlib_resources", "vtk")))


def freeze_float_globals(module):
    """numba freezes a module's float globals as float64 constants."""
    for k, v in list(vars(module).items()):
        if type(v) is float:
            setattr(module, k, np.float64(v))

