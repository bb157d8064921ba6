"""ORACLE — test infrastructure only.

ctypes bindings of
  * the CPU restatement (oracle/_build/liboracle.so, built by oracle/Makefile), and
  * the harness around the reference's own compiled block code
    (oracle/_ref/libswe_ref_s{0,1,2}.so, built by oracle/ref/Makefile from the
    reference sources, only where those sources exist).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker / the timed CPU baseline.

Block state travels as numpy float arrays: the concatenation over blocks
(rank order, block k at (k // blocks_y, k % blocks_y)) of (nx+2)*(ny+2)
values in Float2D layout a[x][y] = raw[x*(ny+2)+y] (src/tools/Float2D.hh:74-76).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# the reference's source tree: SWE_REFERENCE_SRC, else the staged copy
# (oracle/ref/stage.sh) under baseline/_ref
REFERENCE_SRC = os.environ.get("SWE_REFERENCE_SRC") or os.path.join(os.path.dirname(HERE), "baseline", "_ref")

# solver ids (same numbering as the product's C-ABI)
FWAVE, AUGRIE, HYBRID, HLLE = 1, 2, 3, 4
SOLVER_NAMES = {"fwave": FWAVE, "augrie": AUGRIE, "hybrid": HYBRID, "hlle": HLLE}
UNSPLIT, SPLIT = 0, 1
SPLIT_DT_MAX, SPLIT_DT_LAST_EDGE = 0, 1
OUTFLOW, WALL, INFLOW, CONNECT, CONNECT_WITHIN_RANK, PASSIVE = range(6)

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for name, fp in (("oracle_solve_edges_f32", _f32p), ("oracle_solve_edges_f64", _f64p)):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [C.c_int, C.c_int64] + [fp] * 11
        L.oracle_domain_create.restype = C.c_void_p
        L.oracle_domain_create.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.c_double, C.c_double, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int,
                                           C.c_double, C.c_double]
        L.oracle_domain_destroy.argtypes = [C.c_void_p]
        for name in ("oracle_domain_set_state_f32", "oracle_domain_get_state_f32",
                     "oracle_domain_set_state_f64", "oracle_domain_get_state_f64"):
            getattr(L, name).argtypes = [C.c_void_p] + [C.c_void_p] * 4
            getattr(L, name).restype = C.c_int
        L.oracle_domain_bathymetry_ghosts.argtypes = [C.c_void_p]
        L.oracle_domain_set_ghost_layers.argtypes = [C.c_void_p]
        L.oracle_domain_step.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_domain_step_parallel.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_domain_advance.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_void_p]
        L.oracle_domain_time.restype = C.c_double
        L.oracle_domain_time.argtypes = [C.c_void_p]
        L.oracle_lts_round_timesteps.argtypes = [_f32p, C.c_int, C.c_float, C.c_int,
                                                 np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]
        L.oracle_domain_clamp_mass.restype = C.c_double
        L.oracle_domain_clamp_mass.argtypes = [C.c_void_p]
        L.oracle_domain_lts_interval.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_domain_lts_iteration.argtypes = [C.c_void_p]
        L.oracle_domain_lts_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_domain_block_max_timestep.restype = C.c_double
        L.oracle_domain_block_max_timestep.argtypes = [C.c_void_p, C.c_int]
        _lib = L
    return _lib


def solve_edges(solver, hL, hR, huL, huR, bL, bR, precision=32):
    """Per-edge net updates (hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed)."""
    dt = np.float32 if precision == 32 else np.float64
    ins = [np.ascontiguousarray(a, dtype=dt) for a in (hL, hR, huL, huR, bL, bR)]
    n = ins[0].size
    outs = [np.empty(n, dtype=dt) for _ in range(5)]
    fn = lib().oracle_solve_edges_f32 if precision == 32 else lib().oracle_solve_edges_f64
    fn(int(solver), n, *ins, *outs)
    return tuple(outs)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Domain:
    """blocks_x x blocks_y blocks (per-column widths nx_cols, per-row heights ny_rows)."""

    def __init__(self, nx_cols, ny_rows, dx, dy, outer=(OUTFLOW,) * 4, solver=HLLE, semantics=UNSPLIT,
                 split_dt_mode=SPLIT_DT_MAX, precision=32, lts_max_timestep=0.0, duration=0.0):
        self.nx_cols = [int(v) for v in nx_cols]
        self.ny_rows = [int(v) for v in ny_rows]
        self.bx, self.by = len(self.nx_cols), len(self.ny_rows)
        self.precision = precision
        nxa = (C.c_int * self.bx)(*self.nx_cols)
        nya = (C.c_int * self.by)(*self.ny_rows)
        oa = (C.c_int * 4)(*[int(v) for v in outer])
        self.h = lib().oracle_domain_create(precision, self.bx, self.by, nxa, nya, float(dx), float(dy), oa,
                                            int(solver), int(semantics), int(split_dt_mode),
                                            float(lts_max_timestep), float(duration))
        self.ncells = sum((self.nx_cols[k // self.by] + 2) * (self.ny_rows[k % self.by] + 2)
                          for k in range(self.bx * self.by))

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_domain_destroy(self.h)
            self.h = None

    def set_state(self, h=None, hu=None, hv=None, b=None, dtype=np.float32):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=dtype).ravel() for a in (h, hu, hv, b)]
        for a in arrs:
            assert a is None or a.size == self.ncells
        fn = lib().oracle_domain_set_state_f32 if dtype == np.float32 else lib().oracle_domain_set_state_f64
        fn(self.h, *[_ptr(a) for a in arrs])

    def get_state(self, dtype=np.float32):
        arrs = [np.empty(self.ncells, dtype=dtype) for _ in range(4)]
        fn = lib().oracle_domain_get_state_f32 if dtype == np.float32 else lib().oracle_domain_get_state_f64
        fn(self.h, *[_ptr(a) for a in arrs])
        return tuple(arrs)

    def bathymetry_ghosts(self):
        lib().oracle_domain_bathymetry_ghosts(self.h)

    def set_ghost_layers(self):
        lib().oracle_domain_set_ghost_layers(self.h)

    def step(self, n=1):
        dts = np.empty(n, dtype=np.float64)
        lib().oracle_domain_step(self.h, int(n), _ptr(dts))
        return dts

    def step_parallel(self, n=1):
        dts = np.empty(n, dtype=np.float64)
        threads = lib().oracle_domain_step_parallel(self.h, int(n), _ptr(dts))
        return dts, threads

    def advance(self, target, max_steps=10 ** 7):
        dts = np.empty(min(max_steps, 10 ** 6), dtype=np.float64)
        n = lib().oracle_domain_advance(self.h, float(target), int(min(max_steps, dts.size)), _ptr(dts))
        return dts[:n]

    @property
    def time(self):
        return lib().oracle_domain_time(self.h)

    @property
    def clamp_mass(self):
        """depth the dry clamp added so far (sum of -h over the cells it reset)"""
        return lib().oracle_domain_clamp_mass(self.h)

    def lts_iteration(self):
        """one inner local-time-stepping iteration (interval end included when it completes one)"""
        return lib().oracle_domain_lts_iteration(self.h)

    def lts_blocks(self):
        """per block: int[8] (received[4], stepSize, stepSizeCounter, timestepCounter, notified), borderTimestep[4]"""
        n = self.bx * self.by
        ints = np.zeros((n, 8), dtype=np.int32)
        border = np.zeros((n, 4), dtype=np.float64)
        lib().oracle_domain_lts_blocks(self.h, _ptr(ints), _ptr(border))
        return ints, border.astype(np.float32)

    def lts_interval(self, max_iterations=100000):
        steps = np.zeros(self.bx * self.by, dtype=np.int32)
        it = lib().oracle_domain_lts_interval(self.h, int(max_iterations), _ptr(steps))
        return it, steps


def lts_round_timesteps(t, max_timestep_local=1.0, max_divisor=1024):
    """getRoundTimestep's step size for each time step in t (src/blocks/SWE_Block.hh:536-555)"""
    t = np.ascontiguousarray(t, dtype=np.float32)
    out = np.zeros(t.size, dtype=np.int32)
    lib().oracle_lts_round_timesteps(t, t.size, float(max_timestep_local), int(max_divisor), out)
    return out


# ---------------------------------------------------------------------------
# reference harness (oracle/_ref), available only where the reference sources are
# ---------------------------------------------------------------------------
_ref_libs = {}


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE_SRC, "src", "blocks"))


def stage_reference():
    """Copy the reference's source tree into baseline/_ref (oracle/ref/stage.sh,
    which knows where the tree lies on the build machine); False where there
    is none to copy."""
    r = subprocess.run(["sh", os.path.join(HERE, "ref", "stage.sh")], capture_output=True, text=True)
    return r.returncode == 0


def build_reference():
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE_SRC], check=True)


def build_reference_perf():
    """The reference's stock overdecomposed driver with its release flags and
    OpenMP (oracle/_ref/perf/swe_benchmark_mpioverdecomp): the CPU baseline."""
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE_SRC, "perf"], check=True)
    return os.path.join(REF_DIR, "perf", "swe_benchmark_mpioverdecomp")


def ref_lib(macro):
    """Harness compiled with WAVE_PROPAGATION_SOLVER=macro (0 HLLEFun, 1 FWave, 2 AugRie)."""
    if macro not in _ref_libs:
        path = os.path.join(REF_DIR, "libswe_ref_s%d.so" % macro)
        if not _ref_libs:
            build_reference()  # make: rebuilds only what the solver headers or harness changed
        L = C.CDLL(path)
        L.ref_init_block.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                     C.c_float, C.c_void_p] + [C.c_void_p] * 4
        L.ref_domain_geometry.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        for name in ("ref_run_unsplit", "ref_run_split"):
            getattr(L, name).argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p] + [C.c_void_p] * 4 + \
                [C.c_int, C.c_void_p]
        L.ref_run_overdecomp.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                         C.c_void_p] + [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_float,
                                                                           C.c_float, C.c_void_p]
        L.ref_solve_edges.argtypes = [C.c_long] + [_f32p] * 11
        _ref_libs[macro] = L
    return _ref_libs[macro]


def ref_init_block(scenario_id, params, nx, ny, dx, dy, ox, oy, bnd):
    p = np.asarray(list(params) + [0.0] * 8, dtype=np.float64)
    b4 = np.asarray(bnd, dtype=np.int32)
    out = [np.empty((nx + 2) * (ny + 2), dtype=np.float32) for _ in range(4)]
    rc = ref_lib(0).ref_init_block(int(scenario_id), _ptr(p), nx, ny, dx, dy, ox, oy, _ptr(b4), *[_ptr(a) for a in out])
    assert rc == 0
    return tuple(out)


def ref_geometry(scenario_id, params, nx, ny):
    p = np.asarray(list(params) + [0.0] * 8, dtype=np.float64)
    out = np.empty(4, dtype=np.float32)
    assert ref_lib(0).ref_domain_geometry(int(scenario_id), _ptr(p), nx, ny, _ptr(out)) == 0
    return out


def ref_run(kind, macro, nx, ny, dx, dy, bnd, h, hu, hv, b, nsteps):
    """kind 'unsplit' (SWE_DimensionalSplittingMpi) or 'split' (SWE_DimensionalSplitting)."""
    arrs = [np.array(a, dtype=np.float32, copy=True) for a in (h, hu, hv, b)]
    dts = np.empty(nsteps, dtype=np.float32)
    b4 = np.asarray(bnd, dtype=np.int32)
    fn = ref_lib(macro).ref_run_unsplit if kind == "unsplit" else ref_lib(macro).ref_run_split
    fn(nx, ny, dx, dy, _ptr(b4), *[_ptr(a) for a in arrs], int(nsteps), _ptr(dts))
    return arrs[0], arrs[1], arrs[2], dts


def ref_run_overdecomp(macro, nx_cols, ny_rows, dx, dy, outer, h, hu, hv, b, nsteps, lts_max_timestep=0.0,
                       duration=0.0):
    arrs = [np.array(a, dtype=np.float32, copy=True) for a in (h, hu, hv, b)]
    dts = np.empty(nsteps, dtype=np.float32)
    nxa = np.asarray(nx_cols, dtype=np.int32)
    nya = np.asarray(ny_rows, dtype=np.int32)
    o4 = np.asarray(outer, dtype=np.int32)
    steps = np.zeros(len(nx_cols) * len(ny_rows), dtype=np.int32)
    ref_lib(macro).ref_run_overdecomp(len(nx_cols), len(ny_rows), _ptr(nxa), _ptr(nya), dx, dy, _ptr(o4),
                                      *[_ptr(a) for a in arrs], int(nsteps), _ptr(dts), float(lts_max_timestep),
                                      float(duration), _ptr(steps))
    return arrs[0], arrs[1], arrs[2], arrs[3], dts, steps


def ref_solve_edges(macro, hL, hR, huL, huR, bL, bR):
    ins = [np.ascontiguousarray(a, dtype=np.float32) for a in (hL, hR, huL, huR, bL, bR)]
    n = ins[0].size
    outs = [np.empty(n, dtype=np.float32) for _ in range(5)]
    ref_lib(macro).ref_solve_edges(n, *ins, *outs)
    return tuple(outs)
