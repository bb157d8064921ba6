"""Python binding (ctypes) of the GB300 block step: the C ABI of
include/swe_gb300.h (device path) and include/swe_gb300_host.h (host set-up).

There is no CPU fallback: every device call goes to the in-tree CUDA library
(_build/libswe_gb300.so) and raises SweGpuError when the library, the GPU or
a CUDA call fails.

Block state travels as float32 numpy arrays in the reference's Float2D layout
(a[x][y] = raw[x*(ny+2)+y], src/tools/Float2D.hh:74-76); for a multi-block
domain the arrays of all blocks are concatenated in rank order (block k at
(k // blocks_y, k % blocks_y), src/examples/swe_mpi.cpp:186-187).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libswe_gb300.so")

FWAVE, AUGRIE, HYBRID, HLLE = 1, 2, 3, 4
SOLVERS = {"fwave": FWAVE, "augrie": AUGRIE, "hybrid": HYBRID, "hlle": HLLE}
UNSPLIT, SPLIT = 0, 1
EXACT, FAST = 0, 1  # arithmetic of the step (swe_gpu_desc.arithmetic)
SPLIT_DT_MAX, SPLIT_DT_LAST_EDGE = 0, 1
OUTFLOW, WALL, INFLOW, CONNECT, CONNECT_WITHIN_RANK, PASSIVE = range(6)

SCENARIO_RADIAL_DAM_BREAK = 0
SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK = 1
SCENARIO_SEA_AT_REST = 2
SCENARIO_HALF_DOMAIN_DRY = 3
SCENARIO_BATHYMETRY_DAM_BREAK = 4
SCENARIO_SPLASHING_POOL = 5
SCENARIO_SPLASHING_CONE = 6
SCENARIO_DAM_BREAK = 10
SCENARIO_TSUNAMI = 11
SCENARIO_SHORELINE = 12

EXPORTED = [
    "swe_gpu_domain_create", "swe_gpu_domain_destroy", "swe_gpu_block_count", "swe_gpu_block_shape",
    "swe_gpu_upload_block", "swe_gpu_download_block", "swe_gpu_upload_domain", "swe_gpu_download_domain", "swe_gpu_exchange_bathymetry", "swe_gpu_set_ghost_layer",
    "swe_gpu_compute_fluxes", "swe_gpu_update_unknowns", "swe_gpu_get_max_timestep", "swe_gpu_step",
    "swe_gpu_advance", "swe_gpu_get_time", "swe_gpu_set_time", "swe_gpu_sync", "swe_gpu_status",
    "swe_gpu_get_stream", "swe_gpu_set_stream", "swe_gpu_last_error", "swe_gpu_version", "swe_gpu_solve_edges", "swe_gpu_step_block_noalloc",
    "swe_gpu_snapshot_slabs_async", "swe_gpu_snapshot_wait", "swe_gpu_alloc_pinned", "swe_gpu_free_pinned",
    "swe_gpu_launch_count", "swe_gpu_speed_pass_stats", "swe_gpu_lts_advance", "swe_gpu_lts_state", "swe_gpu_lts_blocks",
    "swe_gpu_block_steps", "swe_gpu_ensemble_create", "swe_gpu_group_count", "swe_gpu_group_state",
    "swe_gpu_retile", "swe_gpu_autotune", "swe_gpu_fast_pieces", "swe_gpu_lts_round_timesteps",
    "swe_mlp_last_error", "swe_mlp_gemm_check", "swe_mlp_param_count", "swe_mlp_create", "swe_mlp_destroy",
    "swe_mlp_get_params", "swe_mlp_set_params", "swe_mlp_forward", "swe_mlp_solve", "swe_mlp_loss_grad",
    "swe_mlp_train", "swe_gpu_surrogate_step", "swe_gpu_surrogate_edge_count", "swe_gpu_log_edges",
    "swe_mlp_launch_shape", "swe_gpu_upload_domain_async", "swe_gpu_download_domain_async",
    "swe_nc_open", "swe_nc_write_step", "swe_nc_write_step_slabs", "swe_nc_close",
    "swe_host_scenario_geometry", "swe_host_scenario_boundary", "swe_host_init_block", "swe_host_decompose",
]


class SweGpuError(RuntimeError):
    pass


class Desc(C.Structure):
    _fields_ = [("blocks_x", C.c_int), ("blocks_y", C.c_int), ("nx_cols", C.POINTER(C.c_int)),
                ("ny_rows", C.POINTER(C.c_int)), ("dx", C.c_float), ("dy", C.c_float),
                ("boundary", C.c_int * 4), ("solver", C.c_int), ("semantics", C.c_int),
                ("split_dt_mode", C.c_int), ("tile_rows", C.c_int), ("tile_cols", C.c_int), ("device", C.c_int),
                ("kernel_variant", C.c_int), ("speed_pass", C.c_int), ("lts_max_timestep", C.c_float),
                ("duration", C.c_float), ("arithmetic", C.c_int)]


class Instance(C.Structure):
    """one simulation of an ensemble (swe_gpu_instance)"""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dx", C.c_float), ("dy", C.c_float), ("boundary", C.c_int * 4)]


_lib = None


def build(verbose=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("swe_gb300_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)


def lib():
    """The in-tree CUDA library; raises when it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SweGpuError("CUDA library %s is missing: run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.swe_gpu_last_error.restype = C.c_char_p
        L.swe_gpu_domain_create.argtypes = [C.POINTER(Desc), C.POINTER(vp)]
        L.swe_gpu_domain_destroy.argtypes = [vp]
        L.swe_gpu_block_count.argtypes = [vp, C.POINTER(C.c_int)]
        L.swe_gpu_block_shape.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.swe_gpu_upload_block.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
        L.swe_gpu_download_block.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
        L.swe_gpu_upload_domain.argtypes = [vp, vp, vp, vp, vp]
        L.swe_gpu_download_domain.argtypes = [vp, vp, vp, vp, vp]
        L.swe_gpu_upload_domain_async.argtypes = [vp, vp, vp, vp, vp]
        L.swe_gpu_download_domain_async.argtypes = [vp, vp, vp, vp, vp]
        for n in ("swe_gpu_exchange_bathymetry", "swe_gpu_set_ghost_layer", "swe_gpu_compute_fluxes", "swe_gpu_sync"):
            getattr(L, n).argtypes = [vp]
        L.swe_gpu_update_unknowns.argtypes = [vp, C.c_float]
        L.swe_gpu_get_max_timestep.argtypes = [vp, C.POINTER(C.c_float)]
        L.swe_gpu_step.argtypes = [vp, C.c_int]
        L.swe_gpu_advance.argtypes = [vp, C.c_float, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.swe_gpu_get_time.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int)]
        L.swe_gpu_launch_count.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.swe_gpu_speed_pass_stats.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.swe_gpu_fast_pieces.argtypes = [vp, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        L.swe_gpu_lts_round_timesteps.argtypes = [vp, C.c_int, C.c_float, C.c_int, vp, C.c_int]
        L.swe_gpu_lts_advance.argtypes = [vp, C.c_float, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.swe_gpu_lts_state.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_int), vp]
        L.swe_gpu_lts_blocks.argtypes = [vp, vp, vp]
        L.swe_gpu_block_steps.argtypes = [vp, vp]
        L.swe_mlp_last_error.restype = C.c_char_p
        L.swe_mlp_gemm_check.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.swe_mlp_create.argtypes = [C.c_ulonglong, C.POINTER(vp)]
        L.swe_mlp_destroy.argtypes = [vp]
        L.swe_mlp_destroy.restype = None
        L.swe_mlp_get_params.argtypes = [vp, vp]
        L.swe_mlp_launch_shape.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.swe_mlp_set_params.argtypes = [vp, vp]
        L.swe_mlp_forward.argtypes = [vp, C.c_int, vp, vp]
        L.swe_mlp_solve.argtypes = [vp, C.c_int, vp, vp, vp, vp]
        L.swe_mlp_loss_grad.argtypes = [vp, C.c_int, vp, vp, C.POINTER(C.c_float), vp]
        L.swe_mlp_train.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_float, C.c_ulonglong, vp]
        L.swe_gpu_surrogate_step.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_longlong)]
        L.swe_gpu_surrogate_edge_count.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.swe_gpu_log_edges.argtypes = [vp, C.c_int, C.c_int, vp, vp, C.POINTER(C.c_int)]
        L.swe_gpu_ensemble_create.argtypes = [C.POINTER(Instance), C.c_int, C.POINTER(Desc), C.POINTER(vp)]
        L.swe_gpu_group_count.argtypes = [vp, C.POINTER(C.c_int)]
        L.swe_gpu_group_state.argtypes = [vp, vp, vp, vp]
        L.swe_gpu_retile.argtypes = [vp, C.c_int, C.c_int]
        L.swe_gpu_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.swe_gpu_set_time.argtypes = [vp, C.c_float]
        L.swe_gpu_status.argtypes = [vp, C.POINTER(C.c_int)]
        L.swe_gpu_get_stream.argtypes = [vp, C.POINTER(vp)]
        L.swe_gpu_set_stream.argtypes = [vp, vp]
        L.swe_gpu_solve_edges.argtypes = [C.c_int, C.c_longlong] + [vp] * 11 + [vp]
        L.swe_gpu_step_block_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, vp,
                                                 C.c_int] + [vp] * 7 + [vp, vp]
        L.swe_gpu_snapshot_slabs_async.argtypes = [vp, C.c_int, vp, vp, vp]
        L.swe_gpu_snapshot_wait.argtypes = [vp]
        L.swe_gpu_alloc_pinned.argtypes = [C.c_size_t, C.POINTER(vp)]
        L.swe_gpu_free_pinned.argtypes = [vp]
        L.swe_nc_open.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, vp,
                                  C.c_int, C.POINTER(vp)]
        L.swe_nc_write_step.argtypes = [vp, C.c_float, vp, vp, vp, C.c_int]
        L.swe_nc_write_step_slabs.argtypes = [vp, C.c_float, vp, vp, vp]
        L.swe_nc_close.argtypes = [vp]
        L.swe_host_scenario_geometry.argtypes = [C.c_int, vp, C.c_int, C.c_int, vp]
        L.swe_host_scenario_boundary.argtypes = [C.c_int, vp, vp]
        L.swe_host_init_block.argtypes = [C.c_int, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                          C.c_float, vp, vp, vp, vp, vp, C.c_int]
        L.swe_host_decompose.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                         vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise SweGpuError("swe_gpu error %d: %s" % (rc, lib().swe_gpu_last_error().decode()))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _params(params):
    return np.asarray(list(params or []) + [0.0] * 8, dtype=np.float64)[:8]


# ---------------------------------------------------------------------------
# host-side set-up (initScenario, geometry, decomposition)
# ---------------------------------------------------------------------------
def scenario_geometry(scenario, nx, ny, params=None):
    out = np.empty(4, dtype=np.float32)
    p = _params(params)
    if lib().swe_host_scenario_geometry(int(scenario), _p(p), int(nx), int(ny), _p(out)) != 0:
        raise SweGpuError("unknown scenario %r" % scenario)
    return tuple(float(v) for v in out)


def scenario_boundary(scenario, params=None):
    out = np.empty(4, dtype=np.int32)
    p = _params(params)
    if lib().swe_host_scenario_boundary(int(scenario), _p(p), _p(out)) != 0:
        raise SweGpuError("unknown scenario %r" % scenario)
    return [int(v) for v in out]


def init_block(scenario, nx, ny, dx, dy, origin_x, origin_y, bnd, params=None):
    arrs = [np.empty((nx + 2) * (ny + 2), dtype=np.float32) for _ in range(4)]
    b4 = np.asarray(bnd, dtype=np.int32)
    p = _params(params)
    rc = lib().swe_host_init_block(int(scenario), _p(p), nx, ny, dx, dy, origin_x, origin_y, _p(b4),
                                   *[_p(a) for a in arrs], ny + 2)
    if rc != 0:
        raise SweGpuError("init_block failed")
    return tuple(arrs)


def decompose(nx, ny, nblocks, dx, dy, origin_x=0.0, origin_y=0.0):
    bx, by = C.c_int(), C.c_int()
    cols = np.empty(nblocks, dtype=np.int32)
    rows = np.empty(nblocks, dtype=np.int32)
    ox = np.empty(nblocks, dtype=np.float32)
    oy = np.empty(nblocks, dtype=np.float32)
    rc = lib().swe_host_decompose(nx, ny, nblocks, dx, dy, origin_x, origin_y, C.byref(bx), C.byref(by), _p(cols),
                                  _p(rows), _p(ox), _p(oy))
    if rc != 0:
        raise SweGpuError("decompose failed")
    return (list(cols[:bx.value]), list(rows[:by.value]), list(ox[:bx.value]), list(oy[:by.value]))


def init_domain(scenario, nx, ny, nblocks=1, params=None, boundary=None):
    """The drivers' set-up: geometry, decomposition, per-block initScenario
    (neighbour sides CONNECT_WITHIN_RANK).  Returns (geometry dict, h, hu, hv, b)."""
    dx, dy, ox0, oy0 = scenario_geometry(scenario, nx, ny, params)
    outer = boundary if boundary is not None else scenario_boundary(scenario, params)
    cols, rows, oxs, oys = decompose(nx, ny, nblocks, dx, dy, ox0, oy0)
    bx, by = len(cols), len(rows)
    parts = [[], [], [], []]
    for k in range(bx * by):
        px, py = k // by, k % by
        bnd = [CONNECT_WITHIN_RANK if px > 0 else outer[0], CONNECT_WITHIN_RANK if px < bx - 1 else outer[1],
               CONNECT_WITHIN_RANK if py > 0 else outer[2], CONNECT_WITHIN_RANK if py < by - 1 else outer[3]]
        arrs = init_block(scenario, cols[px], rows[py], dx, dy, oxs[px], oys[py], bnd, params)
        for i in range(4):
            parts[i].append(arrs[i])
    geo = dict(dx=dx, dy=dy, nx_cols=cols, ny_rows=rows, boundary=list(outer), origin_x=oxs, origin_y=oys)
    return (geo,) + tuple(np.concatenate(p) for p in parts)


# ---------------------------------------------------------------------------
# device domain
# ---------------------------------------------------------------------------
class Domain:
    """Blocks of one simulation on the GPU (global time step)."""

    def __init__(self, nx_cols, ny_rows, dx, dy, boundary=(OUTFLOW,) * 4, solver=HLLE, semantics=UNSPLIT,
                 split_dt_mode=SPLIT_DT_MAX, tile_rows=0, tile_cols=0, device=0, kernel_variant=0, speed_pass=0,
                 lts_max_timestep=0.0, duration=0.0, arithmetic=0):
        self.nx_cols = [int(v) for v in nx_cols]
        self.ny_rows = [int(v) for v in ny_rows]
        self.bx, self.by = len(self.nx_cols), len(self.ny_rows)
        self._cols = (C.c_int * self.bx)(*self.nx_cols)
        self._rows = (C.c_int * self.by)(*self.ny_rows)
        d = Desc()
        d.blocks_x, d.blocks_y = self.bx, self.by
        d.nx_cols = C.cast(self._cols, C.POINTER(C.c_int))
        d.ny_rows = C.cast(self._rows, C.POINTER(C.c_int))
        d.dx, d.dy = float(dx), float(dy)
        for i in range(4):
            d.boundary[i] = int(boundary[i])
        d.solver, d.semantics, d.split_dt_mode = int(solver), int(semantics), int(split_dt_mode)
        d.tile_rows, d.tile_cols, d.device = int(tile_rows), int(tile_cols), int(device)
        d.kernel_variant = int(kernel_variant)
        d.speed_pass = int(speed_pass)
        d.lts_max_timestep, d.duration = float(lts_max_timestep), float(duration)
        d.arithmetic = int(arithmetic)
        self.handle = C.c_void_p()
        _check(lib().swe_gpu_domain_create(C.byref(d), C.byref(self.handle)))
        self.shapes = [(self.nx_cols[k // self.by], self.ny_rows[k % self.by]) for k in range(self.bx * self.by)]
        self.offsets = np.cumsum([0] + [(nx + 2) * (ny + 2) for nx, ny in self.shapes])
        self.ncells = int(self.offsets[-1])

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib().swe_gpu_domain_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arrs(self, arrs):
        out = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).ravel() for a in arrs]
        for a in out:
            if a is not None and a.size != self.ncells:
                raise SweGpuError("array of %d values, domain has %d" % (a.size, self.ncells))
        return out

    def upload(self, h=None, hu=None, hv=None, b=None):
        """whole-domain upload (all blocks concatenated); None skips a field"""
        _check(lib().swe_gpu_upload_domain(self.handle, *[_p(a) for a in self._arrs((h, hu, hv, b))]))

    def upload_block(self, k, h=None, hu=None, hv=None, b=None):
        nx, ny = self.shapes[k]
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).ravel() for a in (h, hu, hv, b)]
        _check(lib().swe_gpu_upload_block(self.handle, k, *[_p(a) for a in arrs], ny + 2))

    def download(self):
        arrs = [np.empty(self.ncells, dtype=np.float32) for _ in range(4)]
        _check(lib().swe_gpu_download_domain(self.handle, *[_p(a) for a in arrs]))
        return tuple(arrs)

    def download_block(self, k):
        nx, ny = self.shapes[k]
        arrs = [np.empty((nx + 2) * (ny + 2), dtype=np.float32) for _ in range(4)]
        _check(lib().swe_gpu_download_block(self.handle, k, *[_p(a) for a in arrs], ny + 2))
        return tuple(arrs)

    def download_into(self, arrs):
        """download h, hu, hv (and b if a 4th array is given) into preallocated float32 arrays"""
        arrs = list(arrs) + [None] * (4 - len(arrs))
        for a in arrs:
            if a is not None and (a.dtype != np.float32 or a.size != self.ncells or not a.flags.c_contiguous):
                raise SweGpuError("download_into needs contiguous float32 arrays of the domain size")
        _check(lib().swe_gpu_download_domain(self.handle, *[_p(a) for a in arrs]))

    def upload_async(self, h=None, hu=None, hv=None, b=None):
        """asynchronous whole-domain upload from pinned float32 arrays (left
        unchanged until sync())"""
        arrs = [None if a is None else a for a in (h, hu, hv, b)]
        for a in arrs:
            if a is not None and (a.dtype != np.float32 or a.size != self.ncells or not a.flags.c_contiguous):
                raise SweGpuError("upload_async needs contiguous float32 arrays of the domain size")
        _check(lib().swe_gpu_upload_domain_async(self.handle, *[_p(a) for a in arrs]))

    def download_async(self, arrs):
        """asynchronous download of h, hu, hv (and b) into pinned float32 arrays,
        valid after sync(); overlaps the next upload"""
        arrs = list(arrs) + [None] * (4 - len(arrs))
        for a in arrs:
            if a is not None and (a.dtype != np.float32 or a.size != self.ncells or not a.flags.c_contiguous):
                raise SweGpuError("download_async needs contiguous float32 arrays of the domain size")
        _check(lib().swe_gpu_download_domain_async(self.handle, *[_p(a) for a in arrs]))

    def exchange_bathymetry(self):
        _check(lib().swe_gpu_exchange_bathymetry(self.handle))

    def set_ghost_layer(self):
        _check(lib().swe_gpu_set_ghost_layer(self.handle))

    def compute_fluxes(self):
        _check(lib().swe_gpu_compute_fluxes(self.handle))

    def update_unknowns(self, dt=0.0):
        _check(lib().swe_gpu_update_unknowns(self.handle, float(dt)))

    def max_timestep(self):
        v = C.c_float()
        _check(lib().swe_gpu_get_max_timestep(self.handle, C.byref(v)))
        return v.value

    def step(self, n=1):
        _check(lib().swe_gpu_step(self.handle, int(n)))

    def advance(self, t_end, max_steps=1 << 30):
        n, t = C.c_int(), C.c_float()
        _check(lib().swe_gpu_advance(self.handle, float(t_end), int(max_steps), C.byref(n), C.byref(t)))
        return n.value, t.value

    def time(self):
        t, n = C.c_float(), C.c_int()
        _check(lib().swe_gpu_get_time(self.handle, C.byref(t), C.byref(n)))
        return t.value, n.value

    def launch_count(self):
        """kernels this domain has enqueued so far"""
        n = C.c_longlong()
        _check(lib().swe_gpu_launch_count(self.handle, C.byref(n)))
        return n.value

    def lts_advance(self, t_end, max_iterations=1 << 20):
        """local time stepping until the interval start time reaches t_end or
        max_iterations inner iterations ran: (intervals finished, t)"""
        n, t = C.c_int(), C.c_float()
        rc = lib().swe_gpu_lts_advance(self.handle, float(t_end), int(max_iterations), C.byref(n), C.byref(t))
        if rc != 1:  # SWE_GPU_INCOMPLETE: the iteration budget ran out first
            _check(rc)
        return n.value, t.value

    def lts_state(self):
        """(t, intervals, iterations, per-block steps of the last interval)"""
        t, n, it = C.c_float(), C.c_int(), C.c_int()
        steps = np.zeros(self.bx * self.by, dtype=np.int32)
        _check(lib().swe_gpu_lts_state(self.handle, C.byref(t), C.byref(n), C.byref(it), _p(steps)))
        return t.value, n.value, it.value, steps

    def group_state(self):
        """per dt group: (time, last dt, steps)"""
        n = C.c_int()
        _check(lib().swe_gpu_group_count(self.handle, C.byref(n)))
        t = np.zeros(n.value, dtype=np.float32)
        dt = np.zeros(n.value, dtype=np.float32)
        st = np.zeros(n.value, dtype=np.int32)
        _check(lib().swe_gpu_group_state(self.handle, _p(t), _p(dt), _p(st)))
        return t, dt, st

    def retile(self, tile_rows=0, tile_cols=0):
        _check(lib().swe_gpu_retile(self.handle, int(tile_rows), int(tile_cols)))

    def autotune(self, trial_steps=5):
        """times the candidate tile shapes on a copy of the state, keeps the
        fastest: (tile_rows, tile_cols, ms per step)"""
        r, c, ms = C.c_int(), C.c_int(), C.c_float()
        _check(lib().swe_gpu_autotune(self.handle, int(trial_steps), C.byref(r), C.byref(c), C.byref(ms)))
        return r.value, c.value, ms.value

    def surrogate_step(self, surrogate, nsteps=1, count=True):
        """nsteps unsplit steps with the MLP surrogate (a Surrogate; None: the
        augmented solver on every edge through the same kernels); returns the
        number of edges the surrogate solved when count is set"""
        used = C.c_longlong()
        _check(lib().swe_gpu_surrogate_step(self.handle, surrogate.h if surrogate is not None else None, int(nsteps),
                                            C.byref(used) if count else None))
        return used.value if count else None

    def surrogate_edge_count(self):
        n = C.c_longlong()
        _check(lib().swe_gpu_surrogate_edge_count(self.handle, C.byref(n)))
        return n.value

    def log_edges(self, stride=1, capacity=1 << 20):
        """wet edge states of the current state and their augmented-solver net
        updates: (edges 6 x count, targets 4 x count)"""
        e = np.zeros(6 * capacity, np.float32)
        t = np.zeros(4 * capacity, np.float32)
        c = C.c_int()
        _check(lib().swe_gpu_log_edges(self.handle, int(stride), int(capacity), _p(e), _p(t), C.byref(c)))
        n = c.value
        return e[:6 * n].reshape(6, n).copy(), t[:4 * n].reshape(4, n).copy()

    def block_steps(self):
        """update steps each block has executed"""
        out = np.zeros(self.bx * self.by, dtype=np.int64)
        _check(lib().swe_gpu_block_steps(self.handle, _p(out)))
        return out

    def lts_blocks(self):
        """per block: int[8] (layer states LEFT, RIGHT, BOTTOM, TOP, stepSize, stepSizeCounter,
        timestepCounter, notified) and the layers' neighbour times float[4]"""
        n = self.bx * self.by
        ints = np.zeros((n, 8), dtype=np.int32)
        border = np.zeros((n, 4), dtype=np.float32)
        _check(lib().swe_gpu_lts_blocks(self.handle, _p(ints), _p(border)))
        return ints, border

    def speed_pass_stats(self):
        """(bound tiles, tiles the last bounded speed pass evaluated edge by edge)"""
        t, e = C.c_int(), C.c_int()
        _check(lib().swe_gpu_speed_pass_stats(self.handle, C.byref(t), C.byref(e)))
        return t.value, e.value

    def fast_pieces(self):
        """the fast step's pieces: rows of (block, dir, x0, y0, len)"""
        n = C.c_int()
        _check(lib().swe_gpu_fast_pieces(self.handle, None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 5), dtype=np.int32)
        _check(lib().swe_gpu_fast_pieces(self.handle, _p(out), n.value, C.byref(n)))
        return out[:n.value]

    def set_time(self, t):
        _check(lib().swe_gpu_set_time(self.handle, float(t)))

    def sync(self):
        _check(lib().swe_gpu_sync(self.handle))

    def status(self):
        s = C.c_int()
        _check(lib().swe_gpu_status(self.handle, C.byref(s)))
        return s.value

    def stream(self):
        s = C.c_void_p()
        _check(lib().swe_gpu_get_stream(self.handle, C.byref(s)))
        return s.value

    def snapshot_slabs(self, k, bufs):
        """asynchronous big-endian (y, x) interior slabs of block k into 3 host buffers (addresses)"""
        _check(lib().swe_gpu_snapshot_slabs_async(self.handle, int(k), *[C.c_void_p(b) for b in bufs]))

    def snapshot_wait(self):
        _check(lib().swe_gpu_snapshot_wait(self.handle))

    def set_stream(self, stream):
        """launch on an external cudaStream_t (int handle); None = own stream"""
        _check(lib().swe_gpu_set_stream(self.handle, C.c_void_p(stream or 0)))


class Ensemble(Domain):
    """Independent simulations (one block each, own size, cell size,
    boundaries and dt) stepped together in one handle.  Block k = instance k."""

    def __init__(self, instances, solver=HLLE, semantics=UNSPLIT, split_dt_mode=SPLIT_DT_MAX, tile_rows=0,
                 tile_cols=0, device=0, kernel_variant=0, speed_pass=0, arithmetic=0):
        n = len(instances)
        arr = (Instance * n)()
        for i, (nx, ny, dx, dy, bnd) in enumerate(instances):
            arr[i].nx, arr[i].ny, arr[i].dx, arr[i].dy = int(nx), int(ny), float(dx), float(dy)
            for s4 in range(4):
                arr[i].boundary[s4] = int(bnd[s4])
        d = Desc()
        d.solver, d.semantics, d.split_dt_mode = int(solver), int(semantics), int(split_dt_mode)
        d.tile_rows, d.tile_cols, d.device = int(tile_rows), int(tile_cols), int(device)
        d.kernel_variant, d.speed_pass = int(kernel_variant), int(speed_pass)
        d.arithmetic = int(arithmetic)
        self.handle = C.c_void_p()
        _check(lib().swe_gpu_ensemble_create(arr, n, C.byref(d), C.byref(self.handle)))
        self.bx, self.by = n, 1
        self.nx_cols = [int(i[0]) for i in instances]
        self.ny_rows = [int(i[1]) for i in instances]
        self.shapes = [(int(i[0]), int(i[1])) for i in instances]
        self.offsets = np.cumsum([0] + [(nx + 2) * (ny + 2) for nx, ny in self.shapes])
        self.ncells = int(self.offsets[-1])


def _mlp_check(rc):
    if rc != 0:
        raise SweGpuError("swe_mlp error %d: %s" % (rc, lib().swe_mlp_last_error().decode()))


def tc_gemm_check(x, y, mode=0):
    """Tensor-core GEMM of one CTA (BF16 in, FP32 out): mode 0 D = X Y^T
    (X 128 x k, Y n x k), mode 1 D = X^T Y (X 128 x w1, Y 128 x w2; rows >= w1
    undefined), mode 2 D = X Y (X 128 x w1, Y w1 x w2); D has 128 rows."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    w1 = x.shape[1]
    w2 = y.shape[0] if mode == 0 else y.shape[1]
    d = np.zeros((128, w2), dtype=np.float32)
    _mlp_check(lib().swe_mlp_gemm_check(int(mode), w1, w2, _p(x), _p(y), _p(d)))
    return d


def _edges_soa(edges):
    e = np.ascontiguousarray(edges, dtype=np.float32)
    if e.ndim != 2 or e.shape[0] != 6:
        raise ValueError("edges must be a 6 x n array (hL, hR, huL, huR, bL, bR)")
    return e


class Surrogate:
    """MLP surrogate of the augmented Riemann solver (tensor-core forward,
    backward and Adam training on the device)."""

    NPARAMS = 9028

    def __init__(self, seed=0):
        self.h = C.c_void_p()
        _mlp_check(lib().swe_mlp_create(int(seed), C.byref(self.h)))

    def close(self):
        if self.h:
            lib().swe_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launch_shape(self):
        """(SMs, resident inference CTAs per SM)"""
        a, b = C.c_int(), C.c_int()
        _mlp_check(lib().swe_mlp_launch_shape(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    @property
    def params(self):
        p = np.zeros(self.NPARAMS, np.float32)
        _mlp_check(lib().swe_mlp_get_params(self.h, _p(p)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.NPARAMS
        _mlp_check(lib().swe_mlp_set_params(self.h, _p(p)))

    def forward(self, edges):
        e = _edges_soa(edges)
        out = np.zeros((4, e.shape[1]), np.float32)
        _mlp_check(lib().swe_mlp_forward(self.h, e.shape[1], _p(e), _p(out)))
        return out

    def solve(self, edges):
        """net updates (4 x n), max wave speed (n), used-surrogate flags (n)"""
        e = _edges_soa(edges)
        n = e.shape[1]
        upd = np.zeros((4, n), np.float32)
        spd = np.zeros(n, np.float32)
        used = np.zeros(n, np.uint8)
        _mlp_check(lib().swe_mlp_solve(self.h, n, _p(e), _p(upd), _p(spd), _p(used)))
        return upd, spd, used.astype(bool)

    def loss_grad(self, edges, targets):
        e = _edges_soa(edges)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(self.NPARAMS, np.float32)
        loss = C.c_float()
        _mlp_check(lib().swe_mlp_loss_grad(self.h, e.shape[1], _p(e), _p(t), C.byref(loss), _p(g)))
        return loss.value, g

    def train(self, edges, targets, epochs, batch=4096, lr=1e-3, seed=0):
        e = _edges_soa(edges)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        losses = np.zeros(epochs, np.float32)
        _mlp_check(lib().swe_mlp_train(self.h, e.shape[1], _p(e), _p(t), int(epochs), int(batch), float(lr), int(seed),
                                       _p(losses)))
        return losses


def dam_break_ensemble(count, seed, sizes=None, length=1000.0):
    """`count` radial dam breaks on a length x length square, b = 0, outflow
    sides: nx, ny drawn from `sizes` (default 64, 96, ..., 1024), radius
    U(0.05, 0.3) length, inner height U(5, 20) m, outer height U(1, 5) m, all
    from one seed.  Returns (instances for Ensemble, [(h, hu, hv, b)] per instance)."""
    rng = np.random.default_rng(seed)
    sizes = np.arange(64, 1025, 32) if sizes is None else np.asarray(sizes)
    inst, states = [], []
    for _ in range(count):
        nx, ny = int(rng.choice(sizes)), int(rng.choice(sizes))
        radius = float(rng.uniform(0.05, 0.3)) * length
        hin, hout = float(rng.uniform(5.0, 20.0)), float(rng.uniform(1.0, 5.0))
        dx, dy = float(np.float32(length / nx)), float(np.float32(length / ny))
        bnd = [OUTFLOW] * 4
        states.append(init_block(SCENARIO_DAM_BREAK, nx, ny, dx, dy, 0.0, 0.0, bnd,
                                 [length, radius, hin, hout, 0.0, 0.0, 0.0]))
        inst.append((nx, ny, dx, dy, bnd))
    return inst, states


def lts_round_timesteps(t, max_timestep_local=1.0, max_divisor=1024, device=0):
    """the device's getRoundTimestep step size for each time step in t"""
    t = np.ascontiguousarray(t, dtype=np.float32)
    out = np.zeros(t.size, dtype=np.int32)
    _check(lib().swe_gpu_lts_round_timesteps(_p(t), t.size, float(max_timestep_local), int(max_divisor), _p(out),
                                             int(device)))
    return out


def solve_edges_device(solver, ptrs_in, ptrs_out, n, stream=None):
    """Per-edge solver on device pointers (6 inputs, 5 outputs)."""
    _check(lib().swe_gpu_solve_edges(int(solver), int(n), *[C.c_void_p(p) for p in ptrs_in],
                                     *[C.c_void_p(p) for p in ptrs_out], C.c_void_p(stream or 0)))


def step_block_noalloc(solver, semantics, nx, ny, dx, dy, boundary, ld, ins, outs, stream=None, want_dt=True):
    """Allocation-free step of one block on device pointers: ins = (h, hu, hv, b),
    outs = (h_out, hu_out, hv_out); returns dt when want_dt (the call then waits)."""
    bnd = (C.c_int * 4)(*[int(v) for v in boundary])
    dt = C.c_float()
    _check(lib().swe_gpu_step_block_noalloc(int(solver), int(semantics), int(nx), int(ny), float(dx), float(dy),
                                            C.cast(bnd, C.c_void_p), int(ld), *[C.c_void_p(p) for p in ins],
                                            *[C.c_void_p(p) for p in outs], C.byref(dt) if want_dt else None,
                                            C.c_void_p(stream or 0)))
    return dt.value if want_dt else None


class NetCdfWriter:
    """Block snapshot file with the reference writer's layout (ah/hu/hv(time,y,x), b(y,x))."""

    def __init__(self, path, nx, ny, dx, dy, origin_x, origin_y, b):
        self.nx, self.ny = nx, ny
        bb = np.ascontiguousarray(b, dtype=np.float32).ravel()
        self.h = C.c_void_p()
        rc = lib().swe_nc_open(path.encode(), nx, ny, dx, dy, origin_x, origin_y, _p(bb), ny + 2, C.byref(self.h))
        if rc != 0:
            raise SweGpuError("swe_nc_open(%s) failed: %d" % (path, rc))

    def write(self, t, h, hu, hv):
        arrs = [np.ascontiguousarray(a, dtype=np.float32).ravel() for a in (h, hu, hv)]
        if lib().swe_nc_write_step(self.h, float(t), *[_p(a) for a in arrs], self.ny + 2) != 0:
            raise SweGpuError("swe_nc_write_step failed")

    def write_slabs(self, t, h, hu, hv):
        if lib().swe_nc_write_step_slabs(self.h, float(t), *[C.c_void_p(p) for p in (h, hu, hv)]) != 0:
            raise SweGpuError("swe_nc_write_step_slabs failed")

    def close(self):
        if self.h:
            lib().swe_nc_close(self.h)
            self.h = None
