"""GB300-native electromagnetic-shower stepping loop.

Python front end over the C ABI of ``include/celeritas_gb300.h``. The compute
path is the in-tree CUDA library (``_build/libceleritas_gb300.so``, sm_103a);
there is no CPU fallback: every call that needs the device raises if the
library or a GPU is unavailable.

The classes mirror the reference's host API for the stepping loop:
``Params`` <-> ``celeritas::CoreParams`` (built as in celer-sim's
``Runner::build_core_params``), ``Stepper`` <-> ``celeritas::Stepper`` with
``step(primaries)``, ``step()``, ``run()``, ``kill_active()``, and
``Primary``/``StepResult`` <-> ``celeritas::Primary``/``StepperResult``.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from .build import lib_path

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
DATA_DIR = os.path.join(PACKAGE_DIR, "data")


class GbxError(RuntimeError):
    """Error reported by the C ABI."""


class _Primary(ctypes.Structure):
    _fields_ = [
        ("pdg", ctypes.c_int),
        ("energy", ctypes.c_double),
        ("pos", ctypes.c_double * 3),
        ("dir", ctypes.c_double * 3),
        ("time", ctypes.c_double),
        ("event_id", ctypes.c_uint),
    ]


#: FieldDriverOptions members in the order of gbx_field_driver_options
FIELD_OPTION_NAMES = ("minimum_step", "delta_chord", "delta_intersection", "epsilon_step",
                      "epsilon_rel_max", "errcon", "pgrow", "pshrink", "safety",
                      "max_stepping_increase", "max_stepping_decrease", "max_nsteps",
                      "max_substeps")


class _FieldDriverOptions(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_double) for n in FIELD_OPTION_NAMES[:-2]]
                + [("max_nsteps", ctypes.c_int), ("max_substeps", ctypes.c_int)])


class _ParamsOptions(ctypes.Structure):
    _fields_ = [("field_tesla", ctypes.c_double * 3), ("msc", ctypes.c_int),
                ("track_order", ctypes.c_uint), ("rng_per_track", ctypes.c_int),
                ("event_tallies", ctypes.c_int), ("reentrant_looping", ctypes.c_int),
                ("rz_field_file", ctypes.c_char_p), ("brem_combined", ctypes.c_int),
                ("secondary_stack_factor", ctypes.c_double),
                ("field_options", ctypes.POINTER(_FieldDriverOptions)),
                ("initializer_capacity", ctypes.c_uint)]


#: Step data of a hit (GBX_STEP_* bits of the C header, the reference's
#: StepSelection); step, detector and track_id are always recorded
STEP_SELECT = {
    "pre_time": 1 << 0, "pre_pos": 1 << 1, "pre_dir": 1 << 2, "pre_energy": 1 << 3,
    "post_time": 1 << 4, "post_pos": 1 << 5, "post_dir": 1 << 6, "post_energy": 1 << 7,
    "event_id": 1 << 8, "parent_id": 1 << 9, "track_step_count": 1 << 10,
    "step_length": 1 << 11, "particle": 1 << 12, "energy_deposition": 1 << 13,
}
STEP_SELECT_ALL = (1 << 14) - 1
_HIT_UINT = ("step", "detector", "track_id", "event_id", "parent_id", "track_step_count",
             "particle")
_HIT_DOUBLE = ("step_length", "energy_deposition", "pre_time", "pre_pos", "pre_dir",
               "pre_energy", "post_time", "post_pos", "post_dir", "post_energy")
_HIT_VEC3 = ("pre_pos", "pre_dir", "post_pos", "post_dir")


class _StepHits(ctypes.Structure):
    _fields_ = ([("capacity", ctypes.c_size_t)]
                + [(n, ctypes.POINTER(ctypes.c_uint)) for n in _HIT_UINT]
                + [(n, ctypes.POINTER(ctypes.c_double)) for n in _HIT_DOUBLE])


#: Primary generator distributions (GBX_DIST_*, DistributionSelection)
DISTRIBUTIONS = {"delta": 0, "isotropic": 1, "box": 2}


class _GeneratorOptions(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint), ("pdg", ctypes.c_int * 8), ("num_pdg", ctypes.c_uint),
                ("num_events", ctypes.c_uint), ("primaries_per_event", ctypes.c_uint),
                ("energy_distribution", ctypes.c_int), ("energy", ctypes.c_double * 1),
                ("position_distribution", ctypes.c_int), ("position", ctypes.c_double * 6),
                ("direction_distribution", ctypes.c_int), ("direction", ctypes.c_double * 3)]


class _StepResult(ctypes.Structure):
    _fields_ = [
        ("generated", ctypes.c_uint),
        ("queued", ctypes.c_uint),
        ("active", ctypes.c_uint),
        ("alive", ctypes.c_uint),
    ]


@dataclass(frozen=True)
class StepResult:
    generated: int
    queued: int
    active: int
    alive: int

    def __bool__(self):
        return self.queued > 0 or self.alive > 0


_lib = None
_libs: dict[str, ctypes.CDLL] = {}

# (name, restype, argtypes) for every entry point of include/celeritas_gb300.h
_PROTOTYPES = [
    ("gbx_last_error", ctypes.c_char_p, []),
    ("gbx_params_create", ctypes.c_int,
     [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_ParamsOptions),
      ctypes.POINTER(ctypes.c_void_p)]),
    ("gbx_params_destroy", None, [ctypes.c_void_p]),
    ("gbx_params_num_actions", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    ("gbx_params_action_label", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_uint, ctypes.c_char_p, ctypes.c_size_t]),
    ("gbx_params_num_detectors", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    ("gbx_params_detector_label", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_uint, ctypes.c_char_p, ctypes.c_size_t]),
    ("gbx_stepper_create", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("gbx_stepper_destroy", None, [ctypes.c_void_p]),
    ("gbx_stepper_step", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(_Primary), ctypes.c_size_t, ctypes.POINTER(_StepResult)]),
    ("gbx_stepper_run", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.POINTER(_StepResult),
      ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint)]),
    ("gbx_stepper_launch_action", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint]),
    ("gbx_stepper_insert_primaries", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(_Primary), ctypes.c_size_t]),
    ("gbx_stepper_kill_active", ctypes.c_int, [ctypes.c_void_p]),
    ("gbx_stepper_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("gbx_stepper_stream", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("gbx_stepper_step_kernels", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    ("gbx_stepper_set_action_times", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("gbx_stepper_action_times", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint),
      ctypes.c_size_t]),
    ("gbx_stepper_energy_deposition", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]),
    ("gbx_stepper_clear_energy_deposition", ctypes.c_int, [ctypes.c_void_p]),
    ("gbx_stepper_copy_state", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]),
    ("gbx_stepper_state_info", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t),
      ctypes.POINTER(ctypes.c_size_t)]),
    ("gbx_stepper_extend_from_secondaries_static", ctypes.c_int, [ctypes.c_void_p]),
    ("gbx_stepper_reseed", ctypes.c_int, [ctypes.c_void_p, ctypes.c_ulonglong]),
    ("gbx_stepper_set_tuning", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_longlong]),
    ("gbx_stepper_generate_primaries", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(_GeneratorOptions), ctypes.c_uint]),
    ("gbx_stepper_set_step_output", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_uint, ctypes.c_int, ctypes.c_size_t]),
    ("gbx_stepper_read_step_output", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(_StepHits), ctypes.POINTER(ctypes.c_size_t)]),
    ("gbx_stepper_get_tuning", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]),
    ("gbx_stepper_event_live", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint), ctypes.c_size_t]),
    ("gbx_stepper_sorted_action_sizes", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint), ctypes.c_size_t]),
    ("gbx_stepper_event_energy_deposition", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t, ctypes.c_int]),
    ("gbx_stepper_event_detector_energy_deposition", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_uint, ctypes.c_size_t,
      ctypes.c_int]),
    ("gbx_stepper_warm_up", ctypes.c_int, [ctypes.c_void_p]),
    ("gbx_field_driver_options_default", None, [ctypes.POINTER(_FieldDriverOptions)]),
    ("gbx_device_allocations", ctypes.c_int, [ctypes.POINTER(ctypes.c_ulonglong)]),
    ("gbx_libm_evaluate", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
      ctypes.c_size_t]),
]

#: Elementary functions of the FP64 path (GBX_LIBM_* of the C header)
LIBM_FUNCTIONS = ("exp", "log", "sin", "cos", "tanh", "log1p", "expm1", "cbrt")


def libm_evaluate(function: str, x, precision: str = "double") -> np.ndarray:
    """The stepping loop's FP64 elementary function 'function' evaluated on
    the current device for every element of x."""
    lib = load_library(precision=precision)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    ptr = ctypes.POINTER(ctypes.c_double)
    _check(lib, lib.gbx_libm_evaluate(LIBM_FUNCTIONS.index(function), x.ctypes.data_as(ptr),
                                      y.ctypes.data_as(ptr), x.size))
    return y

EXPORTED_SYMBOLS = [name for name, _, _ in _PROTOTYPES]

#: Supported TrackOrder policies (the reference's enumerator values)
TRACK_ORDERS = {"none": 0, "init_charge": 1, "reindex_shuffle": 2, "reindex_status": 3,
                "reindex_particle_type": 4, "reindex_along_step_action": 5,
                "reindex_step_limit_action": 6, "reindex_both_action": 7}

#: GBX_STATIC_SCRATCH_MAX_SLOTS of the C header
STATIC_SCRATCH_MAX_SLOTS = 131072


def load_library(path: str | None = None, precision: str = "double") -> ctypes.CDLL:
    """Load an in-tree CUDA library; raise if it has not been built.

    ``precision`` is "double" (FP64 throughout, bit-exact with the
    reference's FP64 build) or "mixed" (FP32 physics, FP64 positions,
    geometry, field integration, time and tally).
    """
    global _lib
    if precision in _libs:
        return _libs[precision]
    path = path or lib_path(precision)
    if not os.path.exists(path):
        raise GbxError(
            f"GB300 library not built ({path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, restype, argtypes in _PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _libs[precision] = lib
    if precision == "double":
        _lib = lib
    return lib


def _check(lib: ctypes.CDLL, rc: int):
    if rc != 0:
        msg = lib.gbx_last_error().decode()
        raise GbxError(msg or f"GB300 call failed with status {rc}")


def field_map_file(problem: str = "cms") -> str:
    """Path of a committed synthetic R-Z field map ("cms")."""
    return os.path.join(DATA_DIR, f"{problem}.rzmap.txt")


def geometry_path(geometry: str) -> str:
    """The geometry argument of Params and the oracle programs: a built-in
    name ("calo", "cms") as is, a geometry file of the package's data
    directory (name ending in .geo) as its path, any other path as is."""
    if geometry in ("calo", "cms"):
        return geometry
    if geometry.endswith(".geo") and not os.path.isabs(geometry):
        cand = os.path.join(DATA_DIR, geometry)
        if os.path.exists(cand):
            return cand
    return geometry


def physics_file(problem: str) -> str:
    """Path of a committed synthetic physics input ("calo" or "cms")."""
    return os.path.join(DATA_DIR, f"{problem}.physics.txt")


class Params:
    """Problem parameters on the device (celeritas::CoreParams)."""

    def __init__(self, physics: str, geometry: str = "calo",
                 field_tesla=(0.0, 0.0, 0.0), msc: bool = False,
                 track_order: int | str = "none", precision: str = "double",
                 rng_per_track: bool = False, event_tallies: bool = False,
                 reentrant_looping: bool = False, rz_field: str | None = None,
                 brem_combined: bool = False, secondary_stack_factor: float = 0.0,
                 field_options: dict | None = None, initializer_capacity: int = 0):
        lib = load_library(precision=precision)
        self._lib = lib
        self.precision = precision
        handle = ctypes.c_void_p()
        opts = _ParamsOptions()
        for i in range(3):
            opts.field_tesla[i] = float(field_tesla[i])
        opts.msc = int(msc)
        if isinstance(track_order, str):
            track_order = TRACK_ORDERS[track_order]
        opts.track_order = int(track_order)
        opts.rng_per_track = int(rng_per_track)
        opts.event_tallies = int(event_tallies)
        opts.reentrant_looping = int(reentrant_looping)
        self._rz_field = rz_field.encode() if rz_field else None
        opts.rz_field_file = self._rz_field
        opts.brem_combined = int(brem_combined)
        opts.secondary_stack_factor = float(secondary_stack_factor)
        opts.initializer_capacity = int(initializer_capacity)
        if field_options:
            # FieldDriverOptions: the reference's defaults, then the given
            # members (lengths in cm)
            fo = _FieldDriverOptions()
            lib.gbx_field_driver_options_default(ctypes.byref(fo))
            for name, value in field_options.items():
                if name not in FIELD_OPTION_NAMES:
                    raise GbxError(f"unknown field driver option '{name}'")
                setattr(fo, name, int(value) if name.startswith("max_n") or
                        name == "max_substeps" else float(value))
            self._field_options = fo
            opts.field_options = ctypes.pointer(fo)
        _check(lib, lib.gbx_params_create(physics.encode(), geometry_path(geometry).encode(),
                                     ctypes.byref(opts), ctypes.byref(handle)))
        self._handle = handle
        self.geometry = geometry
        self.field_tesla = tuple(field_tesla)
        self.msc = msc
        self.track_order = int(track_order)

    def __del__(self):
        if getattr(self, "_handle", None):
            self._lib.gbx_params_destroy(self._handle)
            self._handle = None

    @property
    def handle(self):
        return self._handle

    def action_labels(self) -> list[str]:
        n = ctypes.c_uint()
        _check(self._lib, self._lib.gbx_params_num_actions(self._handle, ctypes.byref(n)))
        out = []
        buf = ctypes.create_string_buffer(128)
        for i in range(n.value):
            _check(self._lib, self._lib.gbx_params_action_label(self._handle, i, buf, 128))
            out.append(buf.value.decode())
        return out

    def detector_labels(self) -> list[str]:
        n = ctypes.c_uint()
        _check(self._lib, self._lib.gbx_params_num_detectors(self._handle, ctypes.byref(n)))
        out = []
        buf = ctypes.create_string_buffer(128)
        for i in range(n.value):
            _check(self._lib, self._lib.gbx_params_detector_label(self._handle, i, buf, 128))
            out.append(buf.value.decode())
        return out


#: gbx_primary as a numpy record (field offsets of the C struct)
_PRIMARY_RECORD = np.dtype({
    "names": [name for name, _ in _Primary._fields_],
    "formats": ["<i4", "<f8", ("<f8", 3), ("<f8", 3), "<f8", "<u4"],
    "offsets": [getattr(_Primary, name).offset for name, _ in _Primary._fields_],
    "itemsize": ctypes.sizeof(_Primary)})


def make_primary_array(primaries: np.ndarray):
    """Convert a structured primary array (see primaries.PRIMARY_DTYPE)
    into gbx_primary records, column by column."""
    n = len(primaries)
    arr = (_Primary * max(n, 1))()
    rec = np.frombuffer(arr, dtype=_PRIMARY_RECORD, count=max(n, 1))[:n]
    rec["pdg"] = primaries["pdg"]
    rec["energy"] = primaries["energy"]
    rec["pos"] = primaries["pos"]
    rec["dir"] = primaries["dir"]
    rec["time"] = primaries["time"]
    rec["event_id"] = primaries["event"]
    return arr, n


class Stepper:
    """Device track state and step loop (celeritas::Stepper<MemSpace::device>)."""

    def __init__(self, params: Params, num_track_slots: int, seed: int = 0,
                 use_graph: bool = True):
        self.params = params
        self._lib = params._lib
        handle = ctypes.c_void_p()
        _check(self._lib, self._lib.gbx_stepper_create(params.handle, num_track_slots, seed,
                                       int(use_graph), ctypes.byref(handle)))
        self._handle = handle
        self.num_track_slots = num_track_slots

    def __del__(self):
        if getattr(self, "_handle", None):
            self._lib.gbx_stepper_destroy(self._handle)
            self._handle = None

    @staticmethod
    def _result(r: _StepResult) -> StepResult:
        return StepResult(r.generated, r.queued, r.active, r.alive)

    def step(self, primaries: np.ndarray | None = None) -> StepResult:
        res = _StepResult()
        if primaries is not None and len(primaries):
            arr, n = make_primary_array(primaries)
            _check(self._lib, self._lib.gbx_stepper_step(self._handle, arr, n, ctypes.byref(res)))
        else:
            _check(self._lib, self._lib.gbx_stepper_step(self._handle, None, 0, ctypes.byref(res)))
        return self._result(res)

    def run(self, max_steps: int = 1_000_000, batch: int = 32) -> list[StepResult]:
        """Step until empty; per-step results (host reads every 'batch' steps)."""
        cap = max_steps
        out = (_StepResult * cap)()
        n = ctypes.c_uint()
        _check(self._lib, self._lib.gbx_stepper_run(self._handle, max_steps, batch, out, cap, ctypes.byref(n)))
        return [self._result(out[i]) for i in range(min(n.value, cap))]

    def insert_primaries(self, primaries: np.ndarray):
        arr, n = make_primary_array(primaries)
        _check(self._lib, self._lib.gbx_stepper_insert_primaries(self._handle, arr, n))

    def launch_action(self, action_id: int):
        _check(self._lib, self._lib.gbx_stepper_launch_action(self._handle, action_id))

    def synchronize(self):
        _check(self._lib, self._lib.gbx_stepper_synchronize(self._handle))

    def warm_up(self):
        """Stepper::warm_up: one step over the empty state (kernels loaded,
        step graphs captured); the state must hold no tracks."""
        _check(self._lib, self._lib.gbx_stepper_warm_up(self._handle))

    def kill_active(self):
        _check(self._lib, self._lib.gbx_stepper_kill_active(self._handle))

    def reseed(self, event_id: int):
        """Reseed every slot's random state for an event (Stepper::reseed)."""
        _check(self._lib, self._lib.gbx_stepper_reseed(self._handle, int(event_id)))

    def set_tuning(self, **settings):
        """Launch tuning: along_block_size, along_persistent, sort_threshold,
        sort, sort_material, partition_slots."""
        for name, value in settings.items():
            _check(self._lib, self._lib.gbx_stepper_set_tuning(
                self._handle, name.encode(), int(value)))

    def generate_primaries(self, pdg, energy, position=("delta", (0.0, 0.0, 0.0)),
                           direction=("isotropic", ()), num_events: int = 1,
                           primaries_per_event: int = 1, first_event: int = 0,
                           seed: int = 0):
        """Sample primaries on the device for the next step()
        (PrimaryGenerator with PrimaryGeneratorOptions): ``pdg`` codes cycled
        over each event's primaries, ``energy`` a delta in MeV (a number or
        ("delta", (E,))), ``position`` ("delta", (x, y, z)) or ("box", lo +
        hi) in cm, ``direction`` ("delta", (u, v, w)) or ("isotropic", ())."""
        o = _GeneratorOptions()
        pdgs = [int(p) for p in (pdg if hasattr(pdg, "__len__") else [pdg])]
        o.seed = int(seed)
        o.num_pdg = len(pdgs)
        for i, p in enumerate(pdgs[:8]):
            o.pdg[i] = p
        o.num_events = int(num_events)
        o.primaries_per_event = int(primaries_per_event)
        if not isinstance(energy, tuple):
            energy = ("delta", (float(energy),))
        for prefix, (kind, params), size in (("energy", energy, 1), ("position", position, 6),
                                             ("direction", direction, 3)):
            setattr(o, prefix + "_distribution", DISTRIBUTIONS.get(kind, -1))
            arr = getattr(o, prefix)
            for i, v in enumerate(list(params)[:size]):
                arr[i] = float(v)
        _check(self._lib, self._lib.gbx_stepper_generate_primaries(
            self._handle, ctypes.byref(o), int(first_event)))

    def set_step_output(self, selection="all", nonzero_energy_deposition: bool = True,
                        capacity: int = 1 << 20):
        """Collect the hits of every step (StepCollector + DetectorSteps).

        ``selection`` is "all", an int mask of STEP_SELECT bits, or an
        iterable of STEP_SELECT names; ``capacity`` records are held on the
        device between reads (0 turns the output off). Host buffers of the
        same capacity are kept for ``read_step_output``.
        """
        if isinstance(selection, str) and selection == "all":
            mask = STEP_SELECT_ALL
        elif isinstance(selection, int):
            mask = selection
        else:
            mask = 0
            for name in selection:
                mask |= STEP_SELECT[name]
        _check(self._lib, self._lib.gbx_stepper_set_step_output(
            self._handle, mask, int(nonzero_energy_deposition), int(capacity)))
        self._hit_mask = mask
        self._hit_bufs = {}
        if capacity:
            wanted = {"step", "detector", "track_id"} | {
                n for n, b in STEP_SELECT.items() if mask & b}
            for n in _HIT_UINT + _HIT_DOUBLE:
                if n in wanted:
                    shape = (capacity, 3) if n in _HIT_VEC3 else (capacity,)
                    dtype = np.uint32 if n in _HIT_UINT else np.float64
                    self._hit_bufs[n] = np.zeros(shape, dtype=dtype)
        self._hit_capacity = int(capacity)

    def read_step_output(self, copy: bool = True) -> dict:
        """Hits recorded since the last read, as numpy arrays keyed by field;
        positions and directions have shape (n, 3). With ``copy=False`` the
        arrays are views of the stepper's host buffers, valid until the next
        read."""
        bufs = getattr(self, "_hit_bufs", None)
        if not bufs:
            raise GbxError("step output is not enabled")
        hits = _StepHits()
        hits.capacity = self._hit_capacity
        for n, arr in bufs.items():
            ctype = ctypes.c_uint if n in _HIT_UINT else ctypes.c_double
            setattr(hits, n, arr.ctypes.data_as(ctypes.POINTER(ctype)))
        count = ctypes.c_size_t()
        _check(self._lib, self._lib.gbx_stepper_read_step_output(
            self._handle, ctypes.byref(hits), ctypes.byref(count)))
        n = count.value
        return {k: (arr[:n].copy() if copy else arr[:n]) for k, arr in bufs.items()}

    def get_tuning(self, name: str) -> int:
        v = ctypes.c_longlong()
        _check(self._lib, self._lib.gbx_stepper_get_tuning(
            self._handle, name.encode(), ctypes.byref(v)))
        return v.value

    def sorted_action_sizes(self) -> tuple[np.ndarray, np.ndarray]:
        """Tracks per action (by action ID) in the last along-step and
        step-limit action sorts."""
        n = len(self.params.action_labels())
        out = []
        for key in (0, 1):
            v = np.zeros(n, dtype=np.uint32)
            _check(self._lib, self._lib.gbx_stepper_sorted_action_sizes(
                self._handle, key, v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), n))
            out.append(v.astype(np.int64))
        return out[0], out[1]

    def event_live(self, num_events: int) -> np.ndarray:
        """Live tracks (slots + queued initializers) of events [0, n)."""
        out = np.zeros(num_events, dtype=np.uint32)
        _check(self._lib, self._lib.gbx_stepper_event_live(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), num_events))
        return out

    def event_energy_deposition(self, num_events: int, clear: bool = False) -> np.ndarray:
        """Energy deposited in detectors per event [MeV] (event tallies)."""
        out = np.zeros(num_events, dtype=np.float64)
        _check(self._lib, self._lib.gbx_stepper_event_energy_deposition(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            num_events, int(clear)))
        return out

    def event_detector_energy_deposition(self, first_event: int, num_events: int,
                                         clear: bool = False) -> np.ndarray:
        """Energy deposited in each detector per event [MeV], events
        [first_event, first_event + num_events): array [events, detectors]
        (event tallies)."""
        ndet = len(self.params.detector_labels())
        out = np.zeros((num_events, ndet), dtype=np.float64)
        _check(self._lib, self._lib.gbx_stepper_event_detector_energy_deposition(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            first_event, num_events, int(clear)))
        return out

    def extend_from_secondaries_static(self):
        """Extend-from-secondaries with the library's static scratch array.

        Allocates no device memory; the stepper may have at most
        STATIC_SCRATCH_MAX_SLOTS track slots. Calls that overlap on the GPU
        share the array and race.
        """
        _check(self._lib, self._lib.gbx_stepper_extend_from_secondaries_static(self._handle))

    def stream_handle(self) -> int:
        """cudaStream_t of the stepper, as an integer (for event timing)."""
        s = ctypes.c_void_p()
        _check(self._lib, self._lib.gbx_stepper_stream(self._handle, ctypes.byref(s)))
        return s.value or 0

    def step_kernels(self) -> int:
        """Kernel launches in one graph-replayed step."""
        n = ctypes.c_uint()
        _check(self._lib, self._lib.gbx_stepper_step_kernels(self._handle, ctypes.byref(n)))
        return n.value

    def set_action_times(self, enable: bool = True):
        _check(self._lib, self._lib.gbx_stepper_set_action_times(self._handle, int(enable)))

    def action_times(self) -> tuple[np.ndarray, np.ndarray]:
        """Accumulated device ms and launch counts per action ID (then reset)."""
        n = len(self.params.action_labels())
        ms = np.zeros(n, dtype=np.float64)
        nl = np.zeros(n, dtype=np.uint32)
        _check(self._lib, self._lib.gbx_stepper_action_times(
            self._handle, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            nl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), n))
        return ms, nl

    def energy_deposition(self) -> np.ndarray:
        n = len(self.params.detector_labels())
        out = np.zeros(n, dtype=np.float64)
        _check(self._lib, self._lib.gbx_stepper_energy_deposition(
            self._handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n))
        return out

    def clear_energy_deposition(self):
        _check(self._lib, self._lib.gbx_stepper_clear_energy_deposition(self._handle))

    def state_info(self, field: str) -> tuple[int, int]:
        eb = ctypes.c_size_t()
        cnt = ctypes.c_size_t()
        _check(self._lib, self._lib.gbx_stepper_state_info(self._handle, field.encode(),
                                           ctypes.byref(eb), ctypes.byref(cnt)))
        return eb.value, cnt.value

    def get_state(self, field: str, dtype) -> np.ndarray:
        eb, cnt = self.state_info(field)
        out = np.empty(eb * cnt, dtype=np.uint8)
        _check(self._lib, self._lib.gbx_stepper_copy_state(self._handle, field.encode(),
                                           out.ctypes.data_as(ctypes.c_void_p), out.nbytes, 0))
        return out.view(dtype)

    def set_state(self, field: str, data: np.ndarray):
        data = np.ascontiguousarray(data)
        _check(self._lib, self._lib.gbx_stepper_copy_state(self._handle, field.encode(),
                                           data.ctypes.data_as(ctypes.c_void_p), data.nbytes, 1))


def device_allocations(precision: str = "double") -> int:
    """Device allocations (cudaMalloc calls) made so far by the library."""
    lib = load_library(precision=precision)
    n = ctypes.c_ulonglong()
    _check(lib, lib.gbx_device_allocations(ctypes.byref(n)))
    return int(n.value)
