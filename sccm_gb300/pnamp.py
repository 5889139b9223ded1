"""Python host for the PNAMP C ABI (include/pnamp_gpu.h), via ctypes.

Mirrors the reference's per-pair operator, `Kernel4Triaxial(lpr, Nphi1, Nphi2,
NLEV)` (Codes/PNAMP/PNAMP_Kernel3D.f90:1): the module-state inputs it reads
(model space `tnljm`, Hamiltonian `H`, one-body operators `cME1B`, mesh `AMP`/
`PNP`, `Input%Cscale/iscale`) become the context built once by `PnampContext`,
and each call takes the pair's U0, V0, U1, V1 and returns ZRES and the
projected `Kernel%` fields that `post_general` writes (PNAMP_IO.f90:39-96).

Errors: a non-zero return code of the library raises `PnampError` carrying the
code, where the reference `stop`s. There is no CPU fallback: if the compiled
library is missing or no CUDA device is usable, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from .basis import JJMAX, NOBS, Mesh, ModelSpace

PNAMP_OK = 0
PNAMP_ERR_ARG = 1
PNAMP_ERR_CUDA = 2
PNAMP_ERR_NOMEM = 3
PNAMP_ERR_SINGULAR_U = 4
PNAMP_ERR_UNSUPPORTED = 5
PNAMP_ERR_STATE = 6

ST_PIVOT_UNDERFLOW = 1
ST_SINGULAR_T22 = 2
ST_NONFINITE = 4
ST_SINGULAR_U = 8
ST_CONTRACTION = 16

NK = 2 * JJMAX + 1
FIELDS = ("njkk", "hjkk", "nn", "zz", "J2")

_LIBPATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libpnamp_gb300.so")
_lib = None

# Every symbol the public header declares (tests check the library exports them).
EXPORTS = ("pnamp_init", "pnamp_n_euler", "pnamp_pair", "pnamp_batch", "pnamp_batch_device",
           "pnamp_project", "pnamp_project_device", "pnamp_sync", "pnamp_free",
           "pnamp_strerror", "pnamp_version", "pnamp_batch_device_noalloc", "pnamp_set_form",
           "pnamp_project_q", "pnamp_project_q_device", "pnamp_multi_create", "pnamp_multi_schedule",
           "pnamp_multi_launch", "pnamp_multi_items", "pnamp_multi_free", "pnamp_multi_placement",
           "pnamp_set_outputs", "pnamp_batch_items_device", "pnamp_rho1b_blocks", "pnamp_batch_rho1b_device",
           "pnamp_batch_rho1b", "pnamp_project_rho1b", "pnamp_rho2b_layout", "pnamp_rho2b_tables",
           "pnamp_batch_rho2b_device", "pnamp_batch_rho2b", "pnamp_project_rho2b",
           "pnamp_batch_densities_device", "pnamp_batch_densities", "pnamp_set_timing", "pnamp_stage_times")
# arithmetic forms (include/pnamp_gpu.h PNAMP_FORM_*): plain FP64, double-float per-point algebra,
# and the latter with the two-body contraction on the tensor cores as BF16x3 or BF16x6
FORMS = {"fp64": 0, "df64": 1, "tc3": 2, "tc6": 3}
PNAMP_ERR_SCRATCH_LIMIT = 7
PNAMP_ERR_SMALL_NORM = 8


class PnampError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = load_library().pnamp_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{where}: {msg} (code {code})")


class _Space(C.Structure):
    _fields_ = [("nlev", C.c_int), ("nprot", C.c_int), ("nneut", C.c_int),
                ("core_prot", C.c_int), ("core_neut", C.c_int),
                ("t", C.POINTER(C.c_int)), ("n", C.POINTER(C.c_int)), ("l", C.POINTER(C.c_int)),
                ("twoj", C.POINTER(C.c_int)), ("twom", C.POINTER(C.c_int))]


class _Ham(C.Structure):
    _fields_ = [("e0", C.c_double), ("t1b", C.POINTER(C.c_double)), ("nrec", C.c_int),
                ("ka", C.POINTER(C.c_int)), ("kb", C.POINTER(C.c_int)),
                ("kc", C.POINTER(C.c_int)), ("kd", C.POINTER(C.c_int)),
                ("vbar", C.POINTER(C.c_double)), ("q2", C.POINTER(C.c_double))]


class _Mesh(C.Structure):
    _fields_ = [("nalp", C.c_int), ("nbet", C.c_int), ("ngam", C.c_int), ("nfom", C.c_int),
                ("ncosbet", C.c_int),
                ("alpha", C.POINTER(C.c_double)), ("walp", C.POINTER(C.c_double)),
                ("beta", C.POINTER(C.c_double)), ("wbet", C.POINTER(C.c_double)),
                ("gamma", C.POINTER(C.c_double)), ("wgam", C.POINTER(C.c_double)),
                ("cscale", C.c_double), ("iscale", C.c_int)]


class _Kernels(C.Structure):
    _fields_ = [(f, C.POINTER(C.c_double)) for f in ("njkk", "hjkk", "nn", "zz", "j2")]


def load_library(path: str | None = None):
    """Load the compiled library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or _LIBPATH
    if not os.path.exists(p):
        raise RuntimeError(f"PNAMP CUDA library not built ({p}); run sccm_gb300.build.build()")
    lib = C.CDLL(p)
    vp = C.c_void_p
    lib.pnamp_init.argtypes = [C.POINTER(_Space), C.POINTER(_Ham), C.POINTER(_Mesh), C.POINTER(vp)]
    lib.pnamp_n_euler.argtypes = [vp]
    lib.pnamp_set_form.argtypes = [vp, C.c_int]
    lib.pnamp_set_outputs.argtypes = [vp, C.c_int]
    lib.pnamp_rho1b_blocks.argtypes = [vp] + [C.POINTER(C.c_int)] * 5
    lib.pnamp_batch_rho1b_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    lib.pnamp_batch_rho1b.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.pnamp_project_rho1b.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.pnamp_batch_items_device.argtypes = [vp, C.c_int, vp, C.c_longlong, vp, vp, vp, vp, vp]
    lib.pnamp_rho2b_layout.argtypes = [C.POINTER(_Space), C.POINTER(C.c_int)]
    lib.pnamp_rho2b_tables.argtypes = [C.POINTER(_Space), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_uint), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_double)]
    lib.pnamp_batch_rho2b_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    lib.pnamp_batch_rho2b.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.pnamp_project_rho2b.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.pnamp_batch_densities_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp]
    lib.pnamp_batch_densities.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.pnamp_pair.argtypes = [vp] + [C.POINTER(C.c_double)] * 5 + [C.POINTER(C.c_int)]
    lib.pnamp_batch.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_int)]
    lib.pnamp_batch_device.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    lib.pnamp_batch_device_noalloc.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    lib.pnamp_project.argtypes = [vp, C.POINTER(C.c_double), C.c_int, C.POINTER(_Kernels)]
    lib.pnamp_project_device.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp]
    lib.pnamp_project_q.argtypes = [vp, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]
    lib.pnamp_project_q_device.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp]
    lib.pnamp_multi_create.argtypes = [C.c_int, C.POINTER(vp), C.POINTER(C.c_int), C.POINTER(vp),
                                       C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
    lib.pnamp_multi_schedule.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    lib.pnamp_multi_launch.argtypes = [vp, vp]
    lib.pnamp_multi_placement.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    lib.pnamp_multi_items.argtypes = [vp]
    lib.pnamp_multi_free.argtypes = [vp]
    lib.pnamp_multi_free.restype = None
    lib.pnamp_sync.argtypes = [vp]
    lib.pnamp_set_timing.argtypes = [vp, C.c_int]
    lib.pnamp_stage_times.argtypes = [vp, vp]
    lib.pnamp_free.argtypes = [vp]
    lib.pnamp_free.restype = None
    lib.pnamp_strerror.argtypes = [C.c_int]
    lib.pnamp_strerror.restype = C.c_char_p
    lib.pnamp_version.restype = C.c_char_p
    _lib = lib
    return lib


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class PairResult:
    zres: np.ndarray      # [P_E, NOBS] complex, ZRES(iang, io)
    status: np.ndarray    # [P_E] int bit flags


def rho2b_tables(sp: ModelSpace):
    """Two-particle blocks and m-sum terms of the two-body density (pnamp_rho2b_layout /
    pnamp_rho2b_tables; host only, no device needed).

    Returns dict: blocks [(tt, PP, J, [(o1, o2), ...])] in Write_ME2B's block order,
    quads [nq, 4] levels (k_i, k_j, k_k, k_l), ptr [nelem + 1], term_q, term_c."""
    lib = load_library()
    keep = [np.ascontiguousarray(np.asarray(a, dtype=np.int32)) for a in (sp.t, sp.n, sp.l, sp.twoj, sp.twom)]
    space = _Space(sp.nlev, sp.nprot, sp.nneut, sp.core_prot, sp.core_neut, *[_iptr(a) for a in keep])
    sizes = np.zeros(5, dtype=np.int32)
    rc = lib.pnamp_rho2b_layout(C.byref(space), _iptr(sizes))
    if rc != PNAMP_OK:
        raise PnampError(rc, "pnamp_rho2b_layout")
    nb, ns, ne, nq, nt = (int(x) for x in sizes)
    blk = np.zeros((nb, 4), dtype=np.int32)
    st = np.zeros((ns, 2), dtype=np.int32)
    quads = np.zeros(nq, dtype=np.uint32)
    ptr = np.zeros(ne + 1, dtype=np.int32)
    tq = np.zeros(nt, dtype=np.int32)
    tc = np.zeros(nt)
    rc = lib.pnamp_rho2b_tables(C.byref(space), _iptr(blk), _iptr(st),
                                quads.ctypes.data_as(C.POINTER(C.c_uint)), _iptr(ptr), _iptr(tq), _dptr(tc))
    if rc != PNAMP_OK:
        raise PnampError(rc, "pnamp_rho2b_tables")
    blocks, s0 = [], 0
    for tt, pp, J, na in blk:
        blocks.append((int(tt), int(pp), int(J), [tuple(int(x) for x in st[s0 + a]) for a in range(na)]))
        s0 += na
    q4 = np.stack([(quads >> (8 * k)) & 0xFF for k in range(4)], axis=1).astype(np.int64)
    return {"blocks": blocks, "quads": q4, "ptr": ptr, "term_q": tq, "term_c": tc}


def abi_structs(sp: ModelSpace, e0: float, t1b, recs, vbar, mesh: Mesh, q2=None, cscale: float = 1.0,
                iscale: int = 0):
    """The pnamp_space / pnamp_hamiltonian / pnamp_mesh structs of include/pnamp_gpu.h for these
    inputs, and the arrays they point into (keep them alive while the structs are used)."""
    n = sp.nlev
    keep = []

    def ia(x):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.int32))
        keep.append(a)
        return a

    def da(x):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        keep.append(a)
        return a

    space = _Space(n, sp.nprot, sp.nneut, sp.core_prot, sp.core_neut,
                   _iptr(ia(sp.t)), _iptr(ia(sp.n)), _iptr(ia(sp.l)),
                   _iptr(ia(sp.twoj)), _iptr(ia(sp.twom)))
    recs = np.asarray(recs, dtype=np.int32).reshape(-1, 4)
    t1 = da(np.real(np.asarray(t1b)).T)        # column-major
    q = None
    if q2 is not None:
        q = da(np.asarray(q2, dtype=np.float64).transpose(0, 2, 1))   # each block column-major
    ham = _Ham(float(e0), _dptr(t1), int(recs.shape[0]),
               _iptr(ia(recs[:, 0] + 1)), _iptr(ia(recs[:, 1] + 1)),
               _iptr(ia(recs[:, 2] + 1)), _iptr(ia(recs[:, 3] + 1)),
               _dptr(da(vbar)), _dptr(q) if q is not None else None)
    msh = _Mesh(mesh.nalp, mesh.nbet, mesh.ngam, mesh.nfom, mesh.ncosbet,
                _dptr(da(mesh.alpha)), _dptr(da(mesh.walp)),
                _dptr(da(mesh.beta)), _dptr(da(mesh.wbet)),
                _dptr(da(mesh.gamma)), _dptr(da(mesh.wgam)),
                float(cscale), int(iscale))
    return space, ham, msh, keep


class PnampContext:
    """A built PNAMP context: model space + Hamiltonian + mesh on the GPU."""

    def __init__(self, sp: ModelSpace, e0: float, t1b, recs, vbar, mesh: Mesh,
                 q2=None, cscale: float = 1.0, iscale: int = 0, form: str = "fp64"):
        lib = load_library()
        n = sp.nlev
        self.sp, self.mesh, self.n = sp, mesh, n
        self._space, self._ham, self._mesh, keep = abi_structs(sp, e0, t1b, recs, vbar, mesh, q2, cscale, iscale)
        self._keep = keep
        h = C.c_void_p()
        rc = lib.pnamp_init(C.byref(self._space), C.byref(self._ham), C.byref(self._mesh), C.byref(h))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_init")
        self._h = h
        self.n_euler = lib.pnamp_n_euler(h)
        self.set_form(form)

    def set_form(self, form: str):
        """Arithmetic form: "fp64" (plain), "df64" (double-float per-point algebra), "tc3" / "tc6"
        (double-float with the two-body contraction on the tensor cores, BF16x3 / BF16x6)."""
        rc = load_library().pnamp_set_form(self._h, FORMS[form])
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_set_form")
        self.form = form

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            load_library().pnamp_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------------
    @staticmethod
    def pack_pairs(pairs):
        """[(U0, V0, U1, V1), ...] -> float64 [npairs, 4, n, n] in the ABI's column-major order."""
        out = np.empty((len(pairs), 4) + np.shape(pairs[0][0]), dtype=np.float64)
        for k, quad in enumerate(pairs):
            for q in range(4):
                out[k, q] = np.asarray(quad[q], dtype=np.float64).T
        return out

    def batch(self, pairs_or_packed, check=True):
        """Mesh loop for a batch of pairs -> (zres [npairs, P_E, NOBS], status [npairs, P_E])."""
        uv = pairs_or_packed if isinstance(pairs_or_packed, np.ndarray) else self.pack_pairs(pairs_or_packed)
        uv = np.ascontiguousarray(uv, dtype=np.float64)
        npairs = uv.shape[0]
        z = np.zeros((npairs, NOBS, self.n_euler), dtype=np.complex128)
        st = np.zeros((npairs, self.n_euler), dtype=np.int32)
        rc = load_library().pnamp_batch(self._h, npairs, _dptr(uv),
                                        z.ctypes.data_as(C.POINTER(C.c_double)), _iptr(st))
        if rc != PNAMP_OK and (check or rc != PNAMP_ERR_SINGULAR_U):
            raise PnampError(rc, "pnamp_batch")
        return np.ascontiguousarray(z.transpose(0, 2, 1)), st

    def pair(self, U0, V0, U1, V1) -> PairResult:
        """One pair through `pnamp_pair` (host buffers)."""
        n = self.n
        bufs = [np.asfortranarray(np.asarray(x, dtype=np.float64)) for x in (U0, V0, U1, V1)]
        for b in bufs:
            if b.shape != (n, n):
                raise ValueError(f"expected {n}x{n} matrices")
        z = np.zeros((NOBS, self.n_euler), dtype=np.complex128)
        st = np.zeros(self.n_euler, dtype=np.int32)
        rc = load_library().pnamp_pair(self._h, *[_dptr(b) for b in bufs],
                                       z.ctypes.data_as(C.POINTER(C.c_double)), _iptr(st))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_pair")
        return PairResult(np.ascontiguousarray(z.T), st)

    def project(self, zres, chop=True):
        """J/K projection of one pair's ZRES [P_E, NOBS] -> dict field -> [J, K1+6, K2+6]."""
        z = np.ascontiguousarray(np.asarray(zres, dtype=np.complex128).T)   # [NOBS, P_E]
        if z.shape != (NOBS, self.n_euler):
            raise ValueError("zres must be [P_E, NOBS]")
        out = {f: np.zeros((JJMAX + 1, NK, NK), dtype=np.complex128) for f in FIELDS}
        k = _Kernels(*[out[f].ctypes.data_as(C.POINTER(C.c_double)) for f in FIELDS])
        rc = load_library().pnamp_project(self._h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                          1 if chop else 0, C.byref(k))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_project")
        return out

    def project_q(self, zres, exchange=True):
        """Quadrupole reduced elements -> (qpred, qcpred), each [J2, dJ, K1+8, K2+6] complex."""
        z = np.ascontiguousarray(np.asarray(zres, dtype=np.complex128).T)
        if z.shape != (NOBS, self.n_euler):
            raise ValueError("zres must be [P_E, NOBS]")
        qp = np.zeros((JJMAX + 1, 3, 17, 13), dtype=np.complex128)
        qc = np.zeros_like(qp)
        rc = load_library().pnamp_project_q(self._h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                            1 if exchange else 0, qp.ctypes.data_as(C.POINTER(C.c_double)),
                                            qc.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_project_q")
        return qp, qc

    def rho1b_blocks(self):
        """[(it, lj, n1, n2, twoj)] of the one-body density, in Write_ME1B's order."""
        lib = load_library()
        nb = lib.pnamp_rho1b_blocks(self._h, None, None, None, None, None)
        if nb < 0:
            raise PnampError(-nb, "pnamp_rho1b_blocks")
        arrs = [np.zeros(nb, dtype=np.int32) for _ in range(5)]
        lib.pnamp_rho1b_blocks(self._h, *[_iptr(a) for a in arrs])
        return [tuple(int(a[b]) for a in arrs) for b in range(nb)]

    def batch_rho1b(self, pairs_or_packed):
        """-> (zres [npairs, P_E, NOBS], status, rho1b [npairs, nblocks, P_E]) through the host-buffer ABI."""
        uv = pairs_or_packed if isinstance(pairs_or_packed, np.ndarray) else self.pack_pairs(pairs_or_packed)
        uv = np.ascontiguousarray(uv, dtype=np.float64)
        npairs = uv.shape[0]
        nb = len(self.rho1b_blocks())
        z = np.zeros((npairs, NOBS, self.n_euler), dtype=np.complex128)
        st = np.zeros((npairs, self.n_euler), dtype=np.int32)
        r = np.zeros((npairs, nb, self.n_euler), dtype=np.complex128)
        rc = load_library().pnamp_batch_rho1b(self._h, npairs, _dptr(uv), z.ctypes.data_as(C.POINTER(C.c_double)),
                                              _iptr(st), r.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_rho1b")
        return np.ascontiguousarray(z.transpose(0, 2, 1)), st, r

    def project_rho1b(self, zres, rho1b):
        """One pair: zres [P_E, NOBS], rho1b [nblocks, P_E] -> Write_ME1B values [nblocks]."""
        z = np.ascontiguousarray(np.asarray(zres, dtype=np.complex128).T)
        r = np.ascontiguousarray(np.asarray(rho1b, dtype=np.complex128))
        out = np.zeros(r.shape[0])
        rc = load_library().pnamp_project_rho1b(self._h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                                r.ctypes.data_as(C.POINTER(C.c_double)), _dptr(out))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_project_rho1b")
        return out

    def rho2b_tables(self):
        """The context's two-body density tables (see the module-level `rho2b_tables`)."""
        if getattr(self, "_r2", None) is None:
            self._r2 = rho2b_tables(self.sp)
        return self._r2

    def batch_rho2b(self, pairs_or_packed):
        """-> (zres [npairs, P_E, NOBS], status, rho2b [npairs, nquads]) through the host-buffer ABI;
        rho2b = sum_e w_e (gauge mean of N x the quadruple's density product)."""
        uv = pairs_or_packed if isinstance(pairs_or_packed, np.ndarray) else self.pack_pairs(pairs_or_packed)
        uv = np.ascontiguousarray(uv, dtype=np.float64)
        npairs = uv.shape[0]
        nq = self.rho2b_tables()["quads"].shape[0]
        z = np.zeros((npairs, NOBS, self.n_euler), dtype=np.complex128)
        st = np.zeros((npairs, self.n_euler), dtype=np.int32)
        r = np.zeros((npairs, nq), dtype=np.complex128)
        rc = load_library().pnamp_batch_rho2b(self._h, npairs, _dptr(uv), z.ctypes.data_as(C.POINTER(C.c_double)),
                                              _iptr(st), r.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_rho2b")
        return np.ascontiguousarray(z.transpose(0, 2, 1)), st, r

    def batch_densities(self, pairs_or_packed):
        """-> (zres, status, rho1b [npairs, nblocks, P_E], rho2b [npairs, nquads]) from one pass."""
        uv = pairs_or_packed if isinstance(pairs_or_packed, np.ndarray) else self.pack_pairs(pairs_or_packed)
        uv = np.ascontiguousarray(uv, dtype=np.float64)
        npairs = uv.shape[0]
        nb = len(self.rho1b_blocks())
        nq = self.rho2b_tables()["quads"].shape[0]
        z = np.zeros((npairs, NOBS, self.n_euler), dtype=np.complex128)
        st = np.zeros((npairs, self.n_euler), dtype=np.int32)
        r1 = np.zeros((npairs, nb, self.n_euler), dtype=np.complex128)
        r2 = np.zeros((npairs, nq), dtype=np.complex128)
        rc = load_library().pnamp_batch_densities(self._h, npairs, _dptr(uv), z.ctypes.data_as(C.POINTER(C.c_double)),
                                                  _iptr(st), r1.ctypes.data_as(C.POINTER(C.c_double)),
                                                  r2.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_densities")
        return np.ascontiguousarray(z.transpose(0, 2, 1)), st, r1, r2

    def project_rho2b(self, zres, rho2b):
        """One pair: zres [P_E, NOBS], rho2b [nquads] -> complex Rho2BN per element in block order."""
        z = np.ascontiguousarray(np.asarray(zres, dtype=np.complex128).T)
        r = np.ascontiguousarray(np.asarray(rho2b, dtype=np.complex128))
        out = np.zeros(len(self.rho2b_tables()["ptr"]) - 1, dtype=np.complex128)
        rc = load_library().pnamp_project_rho2b(self._h, z.ctypes.data_as(C.POINTER(C.c_double)),
                                                r.ctypes.data_as(C.POINTER(C.c_double)),
                                                out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_project_rho2b")
        return out

    def set_outputs(self, outputs):
        """"all" (19 observables) or "norm" (N(Omega) only) for later batches."""
        rc = load_library().pnamp_set_outputs(self._h, {"all": 0, "norm": 1}[outputs])
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_set_outputs")
        self.outputs = outputs

    # device-pointer entry points (inputs already resident in HBM)
    def batch_items_device(self, npairs, d_uv, nitems, d_items, d_zres, d_status, d_gauge=0, stream=0):
        """Only the listed (pair, Euler point) items; `d_items` is int32 [nitems, 2]; `d_gauge`
        (optional) receives [npairs][P_E][P_G][N re, N im, H/N re, H/N im] float64."""
        rc = load_library().pnamp_batch_items_device(self._h, npairs, C.c_void_p(d_uv), int(nitems),
                                                     C.c_void_p(d_items), C.c_void_p(d_zres),
                                                     C.c_void_p(d_status), C.c_void_p(d_gauge or None),
                                                     C.c_void_p(stream))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_items_device")

    def batch_device(self, npairs, d_uv, d_zres, d_status, stream=0):
        rc = load_library().pnamp_batch_device(self._h, npairs, C.c_void_p(d_uv), C.c_void_p(d_zres),
                                               C.c_void_p(d_status), C.c_void_p(stream))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_device")

    def batch_rho2b_device(self, npairs, d_uv, d_zres, d_status, d_rho2b, stream=0):
        rc = load_library().pnamp_batch_rho2b_device(self._h, npairs, C.c_void_p(d_uv), C.c_void_p(d_zres),
                                                     C.c_void_p(d_status), C.c_void_p(d_rho2b), C.c_void_p(stream))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_batch_rho2b_device")

    def project_device(self, npairs, d_zres, d_out, chop=True, stream=0):
        rc = load_library().pnamp_project_device(self._h, npairs, C.c_void_p(d_zres), 1 if chop else 0,
                                                 C.c_void_p(d_out), C.c_void_p(stream))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_project_device")

    def sync(self):
        rc = load_library().pnamp_sync(self._h)
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_sync")

    def set_timing(self, on=True):
        """Record CUDA events around the launches of later batch calls (pnamp_set_timing)."""
        rc = load_library().pnamp_set_timing(self._h, 1 if on else 0)
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_set_timing")

    def stage_times(self):
        """ms per stage of the batch calls since set_timing or the previous stage_times, summed:
        dict(setup, points, contract, finish)."""
        ms = np.zeros(4)
        rc = load_library().pnamp_stage_times(self._h, ms.ctypes.data)
        if rc != 4:
            raise PnampError(rc, "pnamp_stage_times")
        return dict(zip(("setup", "points", "contract", "finish"), ms.tolist()))


class MultiPlan:
    """Several contexts' pair batches in one persistent launch (`pnamp_multi_*`).

    `parts` is a list of (ctx, npairs, d_uv, d_zres, d_status) with device
    addresses (ints) the caller keeps alive; results land in each context's
    own buffers as `batch_device` writes them ([npairs][NOBS][P_E] complex,
    [npairs][P_E] status). All contexts must be in the same form.
    """

    def __init__(self, parts):
        lib = load_library()
        k = len(parts)
        vp = C.c_void_p
        hs = (vp * k)(*[p[0]._h for p in parts])
        nps = (C.c_int * k)(*[int(p[1]) for p in parts])
        uvs = (vp * k)(*[p[2] for p in parts])
        zs = (vp * k)(*[p[3] for p in parts])
        sts = (vp * k)(*[p[4] for p in parts])
        h = vp()
        rc = lib.pnamp_multi_create(k, hs, nps, uvs, zs, sts, C.byref(h))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_multi_create")
        self._h = h
        self.parts = parts
        self.nitems = lib.pnamp_multi_items(h)
        self.schedule_args = (1, 1, 0)
        self.smem_budget = 0
        self.smem_bytes = None

    def schedule(self, order=1, grab=1, grid=0):
        rc = load_library().pnamp_multi_schedule(self._h, order, grab, grid)
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_multi_schedule")
        self.schedule_args = (order, grab, grid)

    def placement(self, smem_budget=0):
        """Re-place every context's arrays under `smem_budget` bytes per CTA (0: device maximum)."""
        out = C.c_int(0)
        rc = load_library().pnamp_multi_placement(self._h, int(smem_budget), C.byref(out))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_multi_placement")
        self.smem_budget = int(smem_budget)
        self.smem_bytes = out.value
        return out.value

    def launch(self, stream=0):
        rc = load_library().pnamp_multi_launch(self._h, C.c_void_p(stream))
        if rc != PNAMP_OK:
            raise PnampError(rc, "pnamp_multi_launch")

    def close(self):
        if getattr(self, "_h", None):
            load_library().pnamp_multi_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel4triaxial(ctx: PnampContext, U0, V0, U1, V1, chop=True):
    """Per-pair operator with the reference's name: ZRES and the projected Kernel fields."""
    r = ctx.pair(U0, V0, U1, V1)
    return r.zres, ctx.project(r.zres, chop=chop), r.status
