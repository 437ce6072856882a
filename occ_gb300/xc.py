"""ctypes binding of include/occ_xc.h and the OCC-shaped host classes.

Molecule        occ::core::Molecule (positions in Angstrom, atoms() in Bohr;
                src/core/molecule.cpp:115-121)
AOBasis.load    occ::gto::AOBasis::load (src/gto/shell.cpp:499-571): JSON
                basis, general contractions split, Shell::incorporate_shell_norm
DFT             occ::dft::DFT for the XC part: DFT(method, basis, grid),
                compute_vxc(D) (include/occ/dft/dft.h:395-429),
                exchange_correlation_energy() (dft.h:83)
"""
import ctypes as C
import json
import os
from dataclasses import dataclass, field

import numpy as np

FP64 = 0
MIXED = 1

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
ANGSTROM_TO_BOHR = 1.0 / 0.52917721067  # include/occ/core/units.h:7-8


class XCError(RuntimeError):
    """A failed library call; `code` is the OCC_XC_ERR_* status (or None)."""

    def __init__(self, message, code=None):
        super().__init__(message)
        self.code = code


ERR_ARG, ERR_CUDA, ERR_METHOD, ERR_NOMEM, ERR_TIMEOUT, ERR_BUSY = -1, -2, -3, -4, -5, -6


def library_path():
    return os.path.join(_HERE, "lib", "libocc_xc.so")


class _GridSettings(C.Structure):
    _fields_ = [("max_angular_points", C.c_int), ("min_angular_points", C.c_int),
                ("radial_points", C.c_int), ("radial_precision", C.c_double),
                ("reduced_first_row_element_grid", C.c_int),
                ("treutler_alrichs_adjustment", C.c_int), ("pruning_scheme", C.c_int)]


class _BuildSettings(C.Structure):
    _fields_ = [("xc_screening_threshold", C.c_double), ("density_threshold", C.c_double),
                ("leaf_target", C.c_int), ("leaf_min", C.c_int), ("leaf_max", C.c_int)]


class _MolInfo(C.Structure):
    _fields_ = [("nbf", C.c_int), ("natoms", C.c_int), ("nshells", C.c_int), ("deriv", C.c_int),
                ("npoints", C.c_long), ("nleaves", C.c_long), ("flops_per_build", C.c_double),
                ("device_bytes", C.c_double), ("workspace_bytes", C.c_double),
                ("mixed_workspace_bytes", C.c_double), ("resident_bytes", C.c_double)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _TuneResult(C.Structure):
    _fields_ = [("leaf_target", C.c_int), ("leaf_min", C.c_int), ("leaf_max", C.c_int),
                ("vxc_tile_n", C.c_int), ("persistent_ctas", C.c_int),
                ("ms_per_build", C.c_double), ("default_ms_per_build", C.c_double),
                ("max_dexc", C.c_double), ("candidates", C.c_int), ("from_cache", C.c_int)]


class _ServerSettings(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("queue_capacity", C.c_int),
                ("max_batch", C.c_int), ("precision", C.c_int), ("pool_bytes", C.c_double)]


class _ServerStats(C.Structure):
    _fields_ = [("completed", C.c_long), ("failed", C.c_long), ("pending", C.c_long),
                ("ticks", C.c_long), ("sessions_admitted", C.c_long),
                ("sessions_waiting", C.c_long), ("mean_batch", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("admitted_bytes", C.c_double), ("peak_admitted_bytes", C.c_double)]


def library():
    """Load the in-tree CUDA library; fail loudly if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise XCError(f"{path} is missing: build it with `python -m occ_gb300.build`")
    lib = C.CDLL(path)
    lib.occ_xc_last_error.restype = C.c_char_p
    lib.occ_xc_last_error.argtypes = [C.c_void_p]
    lib.occ_xc_context_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.occ_xc_context_destroy.argtypes = [C.c_void_p]
    lib.occ_xc_normalize_shell.argtypes = [C.c_int, C.c_int, _dp, _dp]
    lib.occ_xc_default_grid_settings.argtypes = [C.POINTER(_GridSettings)]
    lib.occ_xc_default_build_settings.argtypes = [C.POINTER(_BuildSettings)]
    lib.occ_xc_molecule_create.argtypes = [
        C.c_void_p, C.c_int, _ip, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp, C.c_int, C.c_char_p,
        C.POINTER(_GridSettings), C.POINTER(_BuildSettings), C.POINTER(C.c_void_p)]
    lib.occ_xc_molecule_destroy.argtypes = [C.c_void_p]
    lib.occ_xc_molecule_info_get.argtypes = [C.c_void_p, C.POINTER(_MolInfo)]
    lib.occ_xc_molecule_grid.argtypes = [C.c_void_p, _dp, _dp]
    lib.occ_xc_compute_vxc.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_int, _dp, _dp, _dp]
    lib.occ_xc_molecular_grid.argtypes = [C.c_int, _ip, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp,
                                          C.c_int, C.POINTER(_GridSettings),
                                          C.POINTER(C.c_long), _dp, _dp]
    lib.occ_xc_molecular_grid_device.argtypes = [C.c_void_p] + lib.occ_xc_molecular_grid.argtypes
    lib.occ_xc_compute_xc_gradient.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_int, _dp, _dp]
    lib.occ_xc_nlc_vv10.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_double, C.c_double,
                                    C.c_int, _dp, _dp]
    lib.occ_xc_nlc_grid_points.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
    lib.occ_xc_nlc_grid.argtypes = [C.c_void_p, _dp, _dp]
    lib.occ_xc_cosx_create.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(_GridSettings),
                                       C.POINTER(C.c_void_p)]
    lib.occ_xc_cosx_destroy.argtypes = [C.c_void_p]
    lib.occ_xc_cosx_set_precision.argtypes = [C.c_void_p, C.c_int]
    lib.occ_xc_cosx_grid_points.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
    lib.occ_xc_cosx_exchange.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp]
    lib.occ_xc_cosx_exchange_unrestricted.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp]
    lib.occ_xc_cosx_exchange_unrestricted_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                                             C.c_void_p, C.c_void_p]
    lib.occ_xc_cosx_exchange_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]
    lib.occ_xc_compute_vxc_unrestricted.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_int, _dp,
                                                    _dp, _dp]
    lib.occ_xc_compute_vxc_unrestricted_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                                           C.c_int, C.c_void_p, C.c_void_p,
                                                           C.c_void_p]
    lib.occ_xc_molecule_set_gradient_workspace_cap.argtypes = [C.c_void_p, C.c_void_p,
                                                               C.c_double]
    lib.occ_xc_compute_xc_gradient_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_int, C.c_void_p, C.c_void_p,
                                                      C.c_void_p]
    lib.occ_xc_compute_xc_gradient_unrestricted.argtypes = [C.c_void_p, C.c_void_p, _dp,
                                                            C.c_int, _dp, _dp]
    lib.occ_xc_compute_xc_gradient_unrestricted_device.argtypes = [
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.occ_xc_compute_vxc_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_void_p, C.c_void_p]
    _vp = C.c_void_p
    _pp = C.POINTER(C.c_void_p)
    lib.occ_xc_batch_create.argtypes = [_vp, C.c_int, _pp, _pp]
    lib.occ_xc_batch_create_capped.argtypes = [_vp, C.c_int, _pp, C.c_double, _pp]
    lib.occ_xc_batch_destroy.argtypes = [_vp]
    lib.occ_xc_batch_buffers.argtypes = [_vp, C.c_int, _pp, _pp, _pp]
    lib.occ_xc_batch_compute.argtypes = [_vp, _vp, C.c_int, _vp]
    lib.occ_xc_batch_check.argtypes = [_vp, _vp, _vp]
    lib.occ_xc_batch_compute_host.argtypes = [_vp, _vp, C.c_int, _pp, _pp, _dp, _dp]
    lib.occ_xc_graph_capture.argtypes = [_vp, _vp, C.c_int, C.c_int, _pp, _pp, _pp, _pp]
    lib.occ_xc_batch_graph_capture.argtypes = [_vp, _vp, C.c_int, _pp]
    lib.occ_xc_graph_launch.argtypes = [_vp, _vp]
    lib.occ_xc_graph_destroy.argtypes = [_vp]
    lib.occ_xc_set_persistent_ctas.argtypes = [_vp, C.c_int]
    lib.occ_xc_set_wait_limit.argtypes = [_vp, C.c_uint]
    _u64 = C.c_uint64
    lib.occ_xc_default_server_settings.argtypes = [C.POINTER(_ServerSettings)]
    lib.occ_xc_server_last_error.restype = C.c_char_p
    lib.occ_xc_server_last_error.argtypes = []
    lib.occ_xc_server_create.argtypes = [C.c_int, C.POINTER(_ServerSettings), _pp]
    lib.occ_xc_server_destroy.argtypes = [_vp]
    lib.occ_xc_server_open.argtypes = [
        _vp, C.c_int, _ip, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp, C.c_int, C.c_char_p,
        C.POINTER(_GridSettings), C.POINTER(_BuildSettings), C.POINTER(_u64)]
    lib.occ_xc_server_submit.argtypes = [_vp, _u64, _dp, C.POINTER(_u64)]
    lib.occ_xc_server_poll.argtypes = [_vp, _u64, _dp, _dp, C.POINTER(C.c_int)]
    lib.occ_xc_server_wait.argtypes = [_vp, _u64, C.c_double, _dp, _dp]
    lib.occ_xc_server_close.argtypes = [_vp, _u64]
    lib.occ_xc_server_pause.argtypes = [_vp, C.c_int]
    lib.occ_xc_server_session_info.argtypes = [_vp, _u64, C.POINTER(_MolInfo),
                                               C.POINTER(C.c_int)]
    lib.occ_xc_server_stats_get.argtypes = [_vp, C.POINTER(_ServerStats)]
    lib.occ_xc_molecule_set_build_settings.argtypes = [_vp, _vp, C.POINTER(_BuildSettings)]
    lib.occ_xc_molecule_autotune.argtypes = [_vp, _vp, C.c_int, _dp, C.c_double, C.c_int,
                                             C.POINTER(_TuneResult)]
    lib.occ_xc_molecule_apply_tuning.argtypes = [_vp, _vp, C.POINTER(_TuneResult)]
    lib.occ_xc_batch_set_density.argtypes = [_vp, _vp, C.c_int, _dp]
    lib.occ_xc_batch_get_result.argtypes = [_vp, _vp, C.c_int, _dp, _dp]
    _LIB = lib
    return lib


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


@dataclass
class Atom:
    atomic_number: int
    x: float  # Bohr
    y: float
    z: float


class Molecule:
    def __init__(self, atomic_numbers, positions_angstrom):
        self.atomic_numbers = np.asarray(atomic_numbers, dtype=np.int32)
        pos = np.asarray(positions_angstrom, dtype=np.float64)
        if pos.shape == (3, len(self.atomic_numbers)) and pos.shape != (3, 3):
            pos = pos.T
        self.positions = pos.reshape(-1, 3)  # Angstrom, one row per atom

    def atoms(self):
        b = self.positions * ANGSTROM_TO_BOHR
        return [Atom(int(z), *map(float, r)) for z, r in zip(self.atomic_numbers, b)]

    def __len__(self):
        return len(self.atomic_numbers)


@dataclass
class Shell:
    l: int
    atom: int
    origin: np.ndarray  # Bohr
    exponents: np.ndarray
    coefficients: np.ndarray  # normalised (incorporate_shell_norm applied)

    def size(self, pure):
        return 2 * self.l + 1 if pure else (self.l + 1) * (self.l + 2) // 2


def _canonical_basis_name(name):
    return name.lower().replace("*", "_st_")


class AOBasis:
    def __init__(self, atoms, shells, name=""):
        self._atoms = atoms
        self.shells = shells
        self.name = name
        self.pure = False  # OCC's AOBasis is Cartesian until set_pure(true)

    @staticmethod
    def load(atoms, name, path=None):
        fname = os.path.join(path or os.path.join(_HERE, "data", "basis"),
                             _canonical_basis_name(name) + ".json")
        if not os.path.exists(fname):
            raise XCError(f"basis set file not found: {fname}")
        with open(fname) as f:
            elements = json.load(f)["elements"]
        lib = library()
        shells = []
        for a, atom in enumerate(atoms):
            key = str(atom.atomic_number)
            if key not in elements:
                raise XCError(f"element {atom.atomic_number} not found in basis {name}")
            for s in elements[key]["electron_shells"]:
                exps = np.array([float(x) for x in s["exponents"]], dtype=np.float64)
                for i, coefs in enumerate(s["coefficients"]):
                    l = s["angular_momentum"][i % len(s["angular_momentum"])]
                    c = np.array([float(x) for x in coefs], dtype=np.float64)
                    rc = lib.occ_xc_normalize_shell(l, len(exps), _ptr(exps), _ptr(c))
                    if rc != 0:
                        raise XCError(f"cannot normalise shell l={l}")
                    shells.append(Shell(l, a, np.array([atom.x, atom.y, atom.z]), exps.copy(), c))
        return AOBasis(atoms, shells, name)

    def set_pure(self, pure=True):
        self.pure = bool(pure)

    def atoms(self):
        return self._atoms

    def nbf(self):
        return sum(s.size(self.pure) for s in self.shells)

    def nsh(self):
        return len(self.shells)

    def first_bf(self):
        out, n = [], 0
        for s in self.shells:
            out.append(n)
            n += s.size(self.pure)
        return out

    def arrays(self):
        """Flat arrays in the C ABI's layout."""
        l = np.array([s.l for s in self.shells], dtype=np.int32)
        atom = np.array([s.atom for s in self.shells], dtype=np.int32)
        nprim = np.array([len(s.exponents) for s in self.shells], dtype=np.int32)
        exps = np.concatenate([s.exponents for s in self.shells]).astype(np.float64)
        coefs = np.concatenate([s.coefficients for s in self.shells]).astype(np.float64)
        return l, atom, nprim, exps, coefs


@dataclass
class GridSettings:
    """occ::numint::GridSettings defaults (grid_settings.h:81-95)."""
    max_angular_points: int = 302
    min_angular_points: int = 110
    radial_points: int = 50
    radial_precision: float = 1e-12
    reduced_first_row_element_grid: bool = True
    treutler_alrichs_adjustment: bool = True
    pruning_scheme: int = 1

    @staticmethod
    def for_sgx(angular_points=50):
        """GridSettings::for_sgx (src/numint/grid_settings.cpp:59-68): the
        same angular order on every shell, LMG radial precision 1e-5, no
        pruning, no reduced H / He grid."""
        return GridSettings(max_angular_points=angular_points, min_angular_points=angular_points,
                            radial_precision=1e-5, reduced_first_row_element_grid=False,
                            pruning_scheme=0)

    def _c(self):
        return _GridSettings(self.max_angular_points, self.min_angular_points, self.radial_points,
                             self.radial_precision, int(self.reduced_first_row_element_grid),
                             int(self.treutler_alrichs_adjustment), self.pruning_scheme)


@dataclass
class BuildSettings:
    xc_screening_threshold: float = 1e-10
    density_threshold: float = 1e-10
    leaf_target: int = 128
    leaf_min: int = 32
    leaf_max: int = 256

    def _c(self):
        return _BuildSettings(self.xc_screening_threshold, self.density_threshold,
                              self.leaf_target, self.leaf_min, self.leaf_max)


class _Context:
    def __init__(self, device=0):
        lib = library()
        h = C.c_void_p()
        rc = lib.occ_xc_context_create(device, C.byref(h))
        if rc != 0:
            raise XCError(f"occ_xc_context_create failed ({rc})")
        self.h = h
        self.lib = lib

    def error(self):
        return self.lib.occ_xc_last_error(self.h).decode()


# One context per device for the life of the process (never destroyed from
# Python: molecules may be finalised after it at interpreter exit).
_CONTEXTS = {}


def _context(device):
    if device not in _CONTEXTS:
        _CONTEXTS[device] = _Context(device)
    return _CONTEXTS[device]


def molecular_grid(basis, grid_settings=None, device=None):
    """MolecularGrid(basis, settings).get_molecular_grid_points()
    (src/numint/molecular_grid.cpp:11-140): points (N x 3, Bohr) and weights
    in OCC's atom-block layout.  device=None: the host restatement (OpenMP);
    a device index: the Becke partition on that GPU."""
    lib = library()
    atoms = basis.atoms()
    Z = np.array([a.atomic_number for a in atoms], dtype=np.int32)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms], dtype=np.float64).ravel()
    l, at, npr, ex, co = basis.arrays()
    gs = (grid_settings or GridSettings())._c()
    n = C.c_long(0)
    args = (len(Z), _ptr(Z, _ip), _ptr(xyz), len(l), _ptr(l, _ip), _ptr(at, _ip),
            _ptr(npr, _ip), _ptr(ex), _ptr(co), int(basis.pure), C.byref(gs), C.byref(n))
    if device is None:
        fn, pre = lib.occ_xc_molecular_grid, ()
    else:
        ctx = _context(device)
        fn, pre = lib.occ_xc_molecular_grid_device, (ctx.h,)
    rc = fn(*pre, *args, None, None)
    if rc != 0:
        raise XCError(f"molecular grid failed ({rc})", rc)
    P = np.zeros((n.value, 3))
    W = np.zeros(n.value)
    rc = fn(*pre, *args, _ptr(P), _ptr(W))
    if rc != 0:
        raise XCError(f"molecular grid failed ({rc})", rc)
    return P, W


def _molecule_args(method, basis, grid_settings=None, build_settings=None):
    """The molecule arguments of occ_xc_molecule_create / occ_xc_server_open,
    and the arrays they point into (kept alive by the caller)."""
    atoms = basis.atoms()
    Z = np.array([a.atomic_number for a in atoms], dtype=np.int32)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms], dtype=np.float64).ravel()
    l, atom, nprim, exps, coefs = basis.arrays()
    gs = (grid_settings or GridSettings())._c()
    bs = (build_settings or BuildSettings())._c()
    args = (len(Z), _ptr(Z, _ip), _ptr(xyz), len(l), _ptr(l, _ip), _ptr(atom, _ip),
            _ptr(nprim, _ip), _ptr(exps), _ptr(coefs), int(basis.pure), method.encode(),
            C.byref(gs), C.byref(bs))
    return args, (Z, xyz, l, atom, nprim, exps, coefs, gs, bs)


class DFT:
    """The XC part of occ::dft::DFT on one GB300."""

    def __init__(self, method, basis, grid_settings=None, build_settings=None, device=0):
        self.method = method
        self.basis = basis
        self.ctx = _context(device)
        lib = self.ctx.lib
        args, self._keep = _molecule_args(method, basis, grid_settings, build_settings)
        h = C.c_void_p()
        rc = lib.occ_xc_molecule_create(self.ctx.h, *args, C.byref(h))
        if rc != 0:
            raise XCError(f"occ_xc_molecule_create failed ({rc}): {self.ctx.error()}")
        self.h = h
        self._exc = 0.0
        self._nelec = 0.0

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.lib.occ_xc_molecule_destroy(self.h)
            self.h = None

    def info(self):
        i = _MolInfo()
        self.ctx.lib.occ_xc_molecule_info_get(self.h, C.byref(i))
        return {f: getattr(i, f) for f, _ in _MolInfo._fields_}

    def nbf(self):
        return self.basis.nbf()

    def grid(self):
        """(points[N,3] Bohr, weights[N]) in OCC's atom-block layout."""
        n = self.info()["npoints"]
        pts = np.zeros((n, 3))
        w = np.zeros(n)
        self.ctx.lib.occ_xc_molecule_grid(self.h, _ptr(pts), _ptr(w))
        return pts, w

    def compute_vxc(self, D, precision=FP64, out=None):
        """V_xc for mo.D; E_xc via exchange_correlation_energy().  As OCC's
        compute_vxc dispatches on mo.kind, the shape of D decides: nbf x nbf is
        restricted, 2 nbf x nbf (alpha block above beta) unrestricted.  out
        (optional): a Fortran-ordered float64 nbf x nbf array to receive V,
        e.g. in pinned memory."""
        nbf = self.nbf()
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if Dm.shape == (2 * nbf, nbf):
            return self.compute_vxc_unrestricted(Dm, precision)
        if Dm.shape != (nbf, nbf):
            raise XCError(f"density matrix must be {nbf}x{nbf} or {2 * nbf}x{nbf}")
        if out is not None:
            if (out.shape != (nbf, nbf) or out.dtype != np.float64
                    or not out.flags["F_CONTIGUOUS"]):
                raise XCError(f"out must be a Fortran-ordered float64 {nbf}x{nbf} array")
            V = out
        else:
            V = np.zeros((nbf, nbf), order="F")
        exc = C.c_double()
        nel = C.c_double()
        rc = self.ctx.lib.occ_xc_compute_vxc(self.ctx.h, self.h, _ptr(Dm), int(precision),
                                             _ptr(V), C.byref(exc), C.byref(nel))
        if rc != 0:
            raise XCError(f"occ_xc_compute_vxc failed ({rc}): {self.ctx.error()}")
        self._exc = exc.value
        self._nelec = nel.value
        return V

    def compute_vxc_unrestricted(self, D, precision=FP64):
        """UKS V_xc (2 nbf x nbf, alpha block above beta) for OCC's
        unrestricted mo.D (2 nbf x nbf, each block 0.5 C_s C_s^T); FP64 or
        MIXED."""
        nbf = self.nbf()
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if Dm.shape != (2 * nbf, nbf):
            raise XCError(f"unrestricted density matrix must be {2 * nbf}x{nbf}")
        V = np.zeros((2 * nbf, nbf), order="F")
        exc = C.c_double()
        nel = np.zeros(2)
        rc = self.ctx.lib.occ_xc_compute_vxc_unrestricted(self.ctx.h, self.h, _ptr(Dm),
                                                          int(precision), _ptr(V),
                                                          C.byref(exc), _ptr(nel))
        if rc != 0:
            raise XCError(f"occ_xc_compute_vxc_unrestricted failed ({rc}): {self.ctx.error()}",
                          rc)
        self._exc = exc.value
        self._nelec = float(nel.sum())
        self._nelec_ab = (float(nel[0]), float(nel[1]))
        return V

    def integrated_spin_densities(self):
        """(alpha, beta) electron counts of the last unrestricted build."""
        return self._nelec_ab

    def nlc_vv10(self, D, b=6.0, C_vv10=0.01, want_V=True, precision=FP64):
        """VV10 non-local correlation (NonLocalCorrelationFunctional, the
        post-SCF NLC correction of OCC's "-V" methods): (E_nlc, V or None)
        for mo.D = D, restricted, FP64, on OCC's NLC grid."""
        nbf = self.nbf()
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if Dm.shape != (nbf, nbf):
            raise XCError(f"density matrix must be {nbf}x{nbf}")
        V = np.zeros((nbf, nbf), order="F") if want_V else None
        e = C.c_double()
        rc = self.ctx.lib.occ_xc_nlc_vv10(self.ctx.h, self.h, _ptr(Dm), float(b), float(C_vv10),
                                          int(precision), C.byref(e),
                                          _ptr(V) if want_V else None)
        if rc != 0:
            raise XCError(f"occ_xc_nlc_vv10 failed ({rc}): {self.ctx.error()}", rc)
        return e.value, V

    def nlc_grid(self):
        """Points (N x 3) and weights of the NLC grid (after nlc_vv10)."""
        n = C.c_long(-1)
        self.ctx.lib.occ_xc_nlc_grid_points(self.h, C.byref(n))
        if n.value < 0:
            raise XCError("the NLC grid is built by the first nlc_vv10 call")
        P = np.zeros((n.value, 3))
        W = np.zeros(n.value)
        self.ctx.lib.occ_xc_nlc_grid(self.h, _ptr(P), _ptr(W))
        return P, W

    def compute_xc_gradient(self, D, precision=FP64):
        """dE_xc/dR (natoms x 3, Hartree/Bohr) for mo.D = D with the grid held
        fixed (DFT::compute_xc_gradient, include/occ/dft/dft.h:599-749);
        precision FP64 or MIXED (contractions on the tensor cores).  As OCC
        dispatches on mo.kind, the shape of D decides: nbf x nbf restricted,
        2 nbf x nbf (alpha block above beta) unrestricted.  E_xc of the
        same density via exchange_correlation_energy()."""
        nbf = self.nbf()
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        natoms = len(self.basis.atoms())
        g = np.zeros((natoms, 3))
        exc = C.c_double()
        if Dm.shape == (2 * nbf, nbf):
            fn, name = (self.ctx.lib.occ_xc_compute_xc_gradient_unrestricted,
                        "occ_xc_compute_xc_gradient_unrestricted")
        elif Dm.shape == (nbf, nbf):
            fn, name = self.ctx.lib.occ_xc_compute_xc_gradient, "occ_xc_compute_xc_gradient"
        else:
            raise XCError(f"density matrix must be {nbf}x{nbf} or {2 * nbf}x{nbf}")
        rc = fn(self.ctx.h, self.h, _ptr(Dm), int(precision), _ptr(g), C.byref(exc))
        if rc != 0:
            raise XCError(f"{name} failed ({rc}): {self.ctx.error()}", rc)
        self._exc = exc.value
        return g

    def set_gradient_workspace_cap(self, nbytes):
        """Leaves are processed in groups whose gradient workspace stays under
        nbytes (0: the default, 8 GiB)."""
        rc = self.ctx.lib.occ_xc_molecule_set_gradient_workspace_cap(self.ctx.h, self.h,
                                                                     float(nbytes))
        if rc != 0:
            raise XCError(f"occ_xc_molecule_set_gradient_workspace_cap failed ({rc}): "
                          f"{self.ctx.error()}", rc)

    def set_build_settings(self, build_settings):
        """New leaves and screening (DFT::set_xc_screening_threshold and the
        Morton leaf sizes); the grid is kept."""
        bs = build_settings._c()
        rc = self.ctx.lib.occ_xc_molecule_set_build_settings(self.ctx.h, self.h, C.byref(bs))
        if rc != 0:
            raise XCError(f"occ_xc_molecule_set_build_settings failed ({rc}): "
                          f"{self.ctx.error()}", rc)

    def autotune(self, D, precision=MIXED, tol_exc=1e-7, apply=True):
        """Time builds at several leaf sizes / tiles and keep the fastest
        (see occ_xc_molecule_autotune); returns the choice and timings."""
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if Dm.shape != (self.nbf(), self.nbf()):
            raise XCError(f"density matrix must be {self.nbf()}x{self.nbf()}")
        r = _TuneResult()
        rc = self.ctx.lib.occ_xc_molecule_autotune(self.ctx.h, self.h, int(precision), _ptr(Dm),
                                                   float(tol_exc), int(bool(apply)), C.byref(r))
        if rc != 0:
            raise XCError(f"occ_xc_molecule_autotune failed ({rc}): {self.ctx.error()}", rc)
        return {f: getattr(r, f) for f, _ in _TuneResult._fields_}

    def apply_tuning(self, tuning):
        """Apply an autotune() result (e.g. of a molecule of the same size)."""
        r = _TuneResult(**{f: tuning[f] for f, _ in _TuneResult._fields_})
        rc = self.ctx.lib.occ_xc_molecule_apply_tuning(self.ctx.h, self.h, C.byref(r))
        if rc != 0:
            raise XCError(f"occ_xc_molecule_apply_tuning failed ({rc}): {self.ctx.error()}", rc)

    def exchange_correlation_energy(self):
        return self._exc

    def integrated_density(self):
        return self._nelec


class SemiNumericalExchange:
    """occ::qm::cosx::SemiNumericalExchange with set_use_esp(true)
    (include/occ/qm/seminumerical_exchange.h:104-118): the seminumerical
    exchange matrix of a restricted density on its own grid
    (GridSettings.for_sgx(50) unless given), on the GPU in FP64 or with the
    ESP integrals in FP32 (precision=MIXED).  `dft` gives
    the basis and the device (its XC grid is not used)."""

    def __init__(self, dft, grid_settings=None, precision=FP64):
        self.dft = dft
        self.ctx = dft.ctx
        gs = (grid_settings or GridSettings.for_sgx(50))._c()
        h = C.c_void_p()
        rc = self.ctx.lib.occ_xc_cosx_create(self.ctx.h, dft.h, C.byref(gs), C.byref(h))
        if rc != 0:
            raise XCError(f"occ_xc_cosx_create failed ({rc}): {self.ctx.error()}", rc)
        self.h = h
        self.set_precision(precision)

    def set_precision(self, precision):
        """FP64, or MIXED: the ESP integrals in FP32 (F, G, K in FP64)."""
        rc = self.ctx.lib.occ_xc_cosx_set_precision(self.h, int(precision))
        if rc != 0:
            raise XCError(f"occ_xc_cosx_set_precision failed ({rc})", rc)

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.lib.occ_xc_cosx_destroy(self.h)
            self.h = None

    def grid_points(self):
        n = C.c_long(-1)
        self.ctx.lib.occ_xc_cosx_grid_points(self.h, C.byref(n))
        return n.value

    def compute_K(self, D):
        """K of mo.D = D, as compute_K(mo): nbf x nbf for a restricted mo,
        2 nbf x nbf (alpha block above beta, each 0.5 C_s C_s^T) for an
        unrestricted one, K in the same shape."""
        nbf = self.dft.nbf()
        Dm = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if Dm.shape == (nbf, nbf):
            fn, name = self.ctx.lib.occ_xc_cosx_exchange, "occ_xc_cosx_exchange"
        elif Dm.shape == (2 * nbf, nbf):
            fn = self.ctx.lib.occ_xc_cosx_exchange_unrestricted
            name = "occ_xc_cosx_exchange_unrestricted"
        else:
            raise XCError(f"density matrix must be {nbf}x{nbf} or {2 * nbf}x{nbf}")
        K = np.zeros(Dm.shape, order="F")
        rc = fn(self.ctx.h, self.h, _ptr(Dm), _ptr(K))
        if rc != 0:
            raise XCError(f"{name} failed ({rc}): {self.ctx.error()}", rc)
        return K

    def compute_K_device(self, d_D, d_K, stream=None, unrestricted=False):
        """The same on device buffers (addresses, column-major), asynchronous
        on `stream`."""
        if unrestricted:
            fn = self.ctx.lib.occ_xc_cosx_exchange_unrestricted_device
            name = "occ_xc_cosx_exchange_unrestricted_device"
        else:
            fn, name = self.ctx.lib.occ_xc_cosx_exchange_device, "occ_xc_cosx_exchange_device"
        rc = fn(self.ctx.h, self.h, C.c_void_p(d_D), C.c_void_p(d_K),
                C.c_void_p(stream) if stream else None)
        if rc != 0:
            raise XCError(f"{name} failed ({rc}): {self.ctx.error()}", rc)


class Batch:
    """Several molecules built together: one persistent launch sequence per
    precision, the molecules' leaves interleaved over the SMs."""

    def __init__(self, dfts, workspace_cap_bytes=0.0):
        if not dfts:
            raise XCError("a batch needs at least one molecule")
        self.dfts = list(dfts)
        self.ctx = self.dfts[0].ctx
        if any(d.ctx is not self.ctx for d in self.dfts):
            raise XCError("every molecule of a batch must be on the same device")
        hs = (C.c_void_p * len(self.dfts))(*[d.h.value for d in self.dfts])
        h = C.c_void_p()
        rc = self.ctx.lib.occ_xc_batch_create_capped(self.ctx.h, len(self.dfts), hs,
                                                     float(workspace_cap_bytes), C.byref(h))
        if rc != 0:
            raise XCError(f"occ_xc_batch_create failed ({rc}): {self.ctx.error()}")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.lib.occ_xc_batch_destroy(self.h)
            self.h = None

    def __len__(self):
        return len(self.dfts)

    def device_buffers(self, i):
        """(D, V, exc2) device addresses of molecule i's batch-owned buffers."""
        d, v, e = C.c_void_p(), C.c_void_p(), C.c_void_p()
        rc = self.ctx.lib.occ_xc_batch_buffers(self.h, i, C.byref(d), C.byref(v), C.byref(e))
        if rc != 0:
            raise XCError(f"occ_xc_batch_buffers failed ({rc})")
        return d.value, v.value, e.value

    def compute_vxc(self, Ds, precision=FP64):
        """V_xc for every molecule; returns (Vs, E_xc array, integrated densities)."""
        if len(Ds) != len(self.dfts):
            raise XCError(f"expected {len(self.dfts)} density matrices")
        Dm, Vs = [], []
        for D, dft in zip(Ds, self.dfts):
            n = dft.nbf()
            a = np.asfortranarray(np.asarray(D, dtype=np.float64))
            if a.shape != (n, n):
                raise XCError(f"density matrix must be {n}x{n}")
            Dm.append(a)
            Vs.append(np.zeros((n, n), order="F"))
        k = len(Dm)
        dp = (C.c_void_p * k)(*[a.ctypes.data for a in Dm])
        vp = (C.c_void_p * k)(*[a.ctypes.data for a in Vs])
        exc = np.zeros(k)
        nel = np.zeros(k)
        rc = self.ctx.lib.occ_xc_batch_compute_host(self.ctx.h, self.h, int(precision), dp, vp,
                                                    _ptr(exc), _ptr(nel))
        if rc != 0:
            raise XCError(f"occ_xc_batch_compute_host failed ({rc}): {self.ctx.error()}")
        return Vs, exc, nel

    def set_density(self, i, D):
        n = self.dfts[i].nbf()
        a = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if a.shape != (n, n):
            raise XCError(f"density matrix must be {n}x{n}")
        rc = self.ctx.lib.occ_xc_batch_set_density(self.ctx.h, self.h, i, _ptr(a))
        if rc != 0:
            raise XCError(f"occ_xc_batch_set_density failed ({rc}): {self.ctx.error()}")

    def result(self, i):
        """(V, E_xc, integrated density) of molecule i from the batch buffers."""
        n = self.dfts[i].nbf()
        V = np.zeros((n, n), order="F")
        e2 = np.zeros(2)
        rc = self.ctx.lib.occ_xc_batch_get_result(self.ctx.h, self.h, i, _ptr(V), _ptr(e2))
        if rc != 0:
            raise XCError(f"occ_xc_batch_get_result failed ({rc}): {self.ctx.error()}")
        return V, e2[0], e2[1]

    def capture_graph(self, precision=MIXED):
        """One build of the whole batch as a CUDA graph over its own buffers."""
        g = C.c_void_p()
        rc = self.ctx.lib.occ_xc_batch_graph_capture(self.ctx.h, self.h, int(precision),
                                                     C.byref(g))
        if rc != 0:
            raise XCError(f"occ_xc_batch_graph_capture failed ({rc}): {self.ctx.error()}")
        return Graph(self.ctx, g, keep=self)

    def check(self, stream=None):
        rc = self.ctx.lib.occ_xc_batch_check(self.ctx.h, self.h, stream)
        if rc != 0:
            raise XCError(f"occ_xc_batch_check failed ({rc}): {self.ctx.error()}")


class Graph:
    """An instantiated CUDA graph of XC builds; launch() replays it."""

    def __init__(self, ctx, h, keep=None):
        self.ctx = ctx
        self.h = h
        self._keep = keep

    def launch(self, stream=None):
        """stream: a cudaStream_t handle (int) or None for the context's."""
        rc = self.ctx.lib.occ_xc_graph_launch(self.h, C.c_void_p(stream) if stream else None)
        if rc != 0:
            raise XCError(f"occ_xc_graph_launch failed ({rc})")

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.lib.occ_xc_graph_destroy(self.h)
            self.h = None


def capture_scf_graph(dft, precision, d_D, d_V, d_exc2):
    """Capture len(d_D) consecutive builds of one molecule (build k reads the
    device matrix at address d_D[k], writes d_V[k] and the two doubles at
    d_exc2[k]) as one CUDA graph."""
    k = len(d_D)
    if not (k == len(d_V) == len(d_exc2)) or k == 0:
        raise XCError("d_D, d_V and d_exc2 need one address per iteration")
    arr = lambda xs: (C.c_void_p * k)(*[int(x) for x in xs])  # noqa: E731
    g = C.c_void_p()
    rc = dft.ctx.lib.occ_xc_graph_capture(dft.ctx.h, dft.h, int(precision), k, arr(d_D),
                                          arr(d_V), arr(d_exc2), C.byref(g))
    if rc != 0:
        raise XCError(f"occ_xc_graph_capture failed ({rc}): {dft.ctx.error()}")
    return Graph(dft.ctx, g, keep=dft)


def set_persistent_ctas(ctas, device=0):
    """CTAs of the persistent tensor-core kernels (0: one per SM)."""
    ctx = _context(device)
    rc = ctx.lib.occ_xc_set_persistent_ctas(ctx.h, int(ctas))
    if rc != 0:
        raise XCError(f"occ_xc_set_persistent_ctas failed ({rc})")


class Server:
    """Serving loop over one GPU: sessions (one per molecule), submitted
    densities, results by ticket; continuous batching and admission against
    a device-memory budget (occ_xc_server_* in include/occ_xc.h)."""

    def __init__(self, device=0, hbm_budget_bytes=150e9, queue_capacity=4096, max_batch=64,
                 precision=MIXED, pool_bytes=0.0):
        self.lib = library()
        cfg = _ServerSettings(float(hbm_budget_bytes), int(queue_capacity), int(max_batch),
                              int(precision), float(pool_bytes))
        h = C.c_void_p()
        rc = self.lib.occ_xc_server_create(device, C.byref(cfg), C.byref(h))
        if rc != 0:
            raise XCError(f"occ_xc_server_create failed ({rc}): {self._err()}")
        self.h = h
        self._nbf = {}

    def _err(self):
        return self.lib.occ_xc_server_last_error().decode()

    def _check(self, rc, what):
        if rc != 0:
            raise XCError(f"{what} failed ({rc}): {self._err()}", rc)

    def open(self, method, basis, grid_settings=None, build_settings=None):
        args, keep = _molecule_args(method, basis, grid_settings, build_settings)
        sid = C.c_uint64()
        self._check(self.lib.occ_xc_server_open(self.h, *args, C.byref(sid)), "open")
        self._nbf[sid.value] = basis.nbf()
        del keep
        return sid.value

    def submit(self, session, D):
        n = self._nbf[session]
        a = np.asfortranarray(np.asarray(D, dtype=np.float64))
        if a.shape != (n, n):
            raise XCError(f"density matrix must be {n}x{n}")
        t = C.c_uint64()
        self._check(self.lib.occ_xc_server_submit(self.h, session, _ptr(a), C.byref(t)),
                    "submit")
        return t.value, n

    def poll(self, ticket):
        """None while running, else (V, E_xc, integrated density)."""
        tid, n = ticket
        V = np.zeros((n, n), order="F")
        e2 = np.zeros(2)
        done = C.c_int(0)
        self._check(self.lib.occ_xc_server_poll(self.h, tid, _ptr(V), _ptr(e2), C.byref(done)),
                    "poll")
        return (V, e2[0], e2[1]) if done.value else None

    def wait(self, ticket, timeout=120.0):
        tid, n = ticket
        V = np.zeros((n, n), order="F")
        e2 = np.zeros(2)
        self._check(self.lib.occ_xc_server_wait(self.h, tid, float(timeout), _ptr(V), _ptr(e2)),
                    "wait")
        return V, e2[0], e2[1]

    def close(self, session):
        self._check(self.lib.occ_xc_server_close(self.h, session), "close")

    def pause(self, paused=True):
        self._check(self.lib.occ_xc_server_pause(self.h, int(bool(paused))), "pause")

    def session_info(self, session):
        i = _MolInfo()
        adm = C.c_int(0)
        self._check(self.lib.occ_xc_server_session_info(self.h, session, C.byref(i),
                                                        C.byref(adm)), "session_info")
        d = {f: getattr(i, f) for f, _ in _MolInfo._fields_}
        d["admitted"] = bool(adm.value)
        return d

    def stats(self):
        st = _ServerStats()
        self._check(self.lib.occ_xc_server_stats_get(self.h, C.byref(st)), "stats")
        return {f: getattr(st, f) for f, _ in _ServerStats._fields_}

    def shutdown(self):
        if getattr(self, "h", None):
            self.lib.occ_xc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.shutdown()
