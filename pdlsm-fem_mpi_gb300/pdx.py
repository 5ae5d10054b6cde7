"""ctypes binding of the C ABI in include/pdx.h (lib/libpdx.so, built in-tree).

This is the reference-facing seam as a Python caller binds it: plain
pointers and sizes, numpy arrays on the host, status codes turned into
exceptions.  Loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpdx.so")

STATUS = {0: "OK", 1: "IO", 2: "PARSE", 3: "UNSUPPORTED", 4: "INVALID", 5: "CUDA", 6: "SINGULAR",
          7: "NOCONV", 8: "NODEVICE", 9: "NUMERIC"}


class PdxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pdx status {STATUS.get(code, code)}: {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("lanes", C.c_int), ("verbose", C.c_int),
                ("fe_lanes", C.c_int)]


class ModelInfo(C.Structure):
    _fields_ = [("dim", C.c_int), ("n_node", C.c_int), ("n_elem", C.c_int), ("n_eq", C.c_int),
                ("n_fam", C.c_int), ("n_pdbe", C.c_int), ("n_fe", C.c_int), ("n_fe_classes", C.c_int),
                ("n_bond", C.c_int64), ("nnz", C.c_int64), ("solver", C.c_int), ("newmark", C.c_int),
                ("lumped", C.c_int), ("fail_flag", C.c_int), ("precision", C.c_int), ("nsteps", C.c_int),
                ("save_freq", C.c_int), ("lanes", C.c_int), ("fe_lanes", C.c_int), ("dt", C.c_double), ("min_delta", C.c_double),
                ("max_delta", C.c_double), ("s0", C.c_double), ("s0_pert", C.c_double)]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("rtol", C.c_double), ("max_iter", C.c_int), ("use_x0", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("seconds", C.c_double),
                ("converged", C.c_int), ("method_used", C.c_int), ("refinements", C.c_int),
                ("setup_seconds", C.c_double)]


EXPORTED = ["pdx_last_error", "pdx_version", "pdx_model_create_from_cmd", "pdx_model_destroy",
            "pdx_model_get_info", "pdx_model_array_len", "pdx_model_array", "pdx_bond_coefficients",
            "pdx_internal_force", "pdx_explicit_init", "pdx_explicit_advance", "pdx_explicit_advance_timed",
            "pdx_explicit_step_host", "pdx_explicit_step_count", "pdx_get_state", "pdx_assemble_csr",
            "pdx_solve_csr", "pdx_run", "pdx_pcg_solve_noalloc", "pdx_batch_create", "pdx_batch_size",
            "pdx_batch_offsets", "pdx_newmark_init", "pdx_newmark_step", "pdx_learned_setup", "pdx_learned_samples",
            "pdx_learned_train", "pdx_mlp_params", "pdx_mlp_loss_grad", "pdx_learned_probe",
            "pdx_learned_pairs", "pdx_learned_options", "pdx_learned_active",
            "pdx_quasi_init", "pdx_quasi_step", "pdx_reaction_forces", "pdx_crack_state", "pdx_crack_advance"]

_lib: Optional[C.CDLL] = None

_P = C.c_void_p
_D = C.POINTER(C.c_double)


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(LIB_PATH)
    L.pdx_last_error.restype = C.c_char_p
    L.pdx_version.restype = C.c_char_p
    L.pdx_model_create_from_cmd.argtypes = [C.c_char_p, C.POINTER(Options), C.POINTER(_P)]
    L.pdx_model_destroy.argtypes = [_P]
    L.pdx_model_destroy.restype = None
    L.pdx_model_get_info.argtypes = [_P, C.POINTER(ModelInfo)]
    L.pdx_model_array_len.argtypes = [_P, C.c_char_p, C.POINTER(C.c_int64)]
    L.pdx_model_array.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.pdx_bond_coefficients.argtypes = [_P, _D, _D, _D, _D]
    L.pdx_internal_force.argtypes = [_P, _D, _D]
    L.pdx_explicit_init.argtypes = [_P]
    L.pdx_explicit_advance.argtypes = [_P, C.c_int]
    L.pdx_explicit_advance_timed.argtypes = [_P, C.c_int, _D]
    L.pdx_explicit_step_host.argtypes = [_P, _D, _D, _D]
    L.pdx_explicit_step_count.argtypes = [_P]
    L.pdx_explicit_step_count.restype = C.c_int64
    L.pdx_get_state.argtypes = [_P, _D, _D, _D, C.POINTER(C.c_uint8)]
    L.pdx_assemble_csr.argtypes = [_P, C.c_int, _D, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _D, _D]
    L.pdx_solve_csr.argtypes = [C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _D, _D, _D,
                                C.POINTER(SolveOpts), C.POINTER(SolveInfo)]
    L.pdx_run.argtypes = [_P, C.c_char_p]
    L.pdx_pcg_solve_noalloc.argtypes = [C.c_int64, C.c_int64, _P, _P, _P, _P, _P, C.POINTER(SolveOpts), _P,
                                        C.POINTER(SolveInfo)]
    _F = C.POINTER(C.c_float)
    for name, args in (("pdx_newmark_init", [_P]),
                       ("pdx_newmark_step", [_P, C.c_int, C.c_int, C.POINTER(SolveInfo)]),
                       ("pdx_learned_setup", [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int]),
                       ("pdx_learned_train", [_P, C.c_int, C.c_float, C.c_uint64, _F]),
                       ("pdx_mlp_params", [_P, _F, _F, C.POINTER(C.c_int64)]),
                       ("pdx_mlp_loss_grad", [_P, C.c_int, _F, _F, _F, _F, _F]),
                       ("pdx_learned_probe", [_P, C.c_int, C.c_uint64]),
                       ("pdx_learned_options", [_P, C.c_int, C.c_int]),
                       ("pdx_quasi_init", [_P]),
                       ("pdx_reaction_forces", [_P, _D, C.c_int64, C.POINTER(C.c_int64)]),
                       ("pdx_quasi_step", [_P, C.c_int, C.POINTER(SolveInfo)]),
                       ("pdx_crack_state", [_P, _D, C.c_int, C.POINTER(C.c_int)]),
                       ("pdx_crack_advance", [_P, _D, C.POINTER(C.c_uint8)]),
                       ("pdx_learned_pairs", [_P, _F, _F, C.POINTER(C.c_int64), C.POINTER(C.c_int)])):
        getattr(L, name).argtypes = args
        getattr(L, name).restype = C.c_int
    L.pdx_learned_active.argtypes = [_P]
    L.pdx_learned_active.restype = C.c_int
    L.pdx_learned_samples.argtypes = [_P]
    L.pdx_learned_samples.restype = C.c_int64
    L.pdx_batch_create.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.POINTER(Options), C.POINTER(_P)]
    L.pdx_batch_create.restype = C.c_int
    L.pdx_batch_size.argtypes = [_P]
    L.pdx_batch_size.restype = C.c_int
    L.pdx_batch_offsets.argtypes = [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.pdx_batch_offsets.restype = C.c_int
    for name in ("pdx_model_create_from_cmd", "pdx_model_get_info", "pdx_model_array_len", "pdx_model_array",
                 "pdx_bond_coefficients", "pdx_internal_force", "pdx_explicit_init", "pdx_explicit_advance",
                 "pdx_explicit_advance_timed", "pdx_explicit_step_host", "pdx_get_state", "pdx_assemble_csr",
                 "pdx_solve_csr", "pdx_run", "pdx_pcg_solve_noalloc"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(code: int) -> None:
    if code != 0:
        raise PdxError(code, lib().pdx_last_error().decode())


def _dptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_D)


_ARRAY_DTYPES = {"eq": np.int32, "vol_node": np.float64, "vol_elem": np.float64, "node_type": np.int32,
                 "fam_off": np.int64, "fam_members": np.int32, "fam_horizon": np.float64, "fam_cdv": np.float64,
                 "bond_state0": np.uint8, "pdbe": np.int32, "pde_idx": np.int32, "fe_idx": np.int32,
                 "csr_ia": np.int64, "csr_ja": np.int64, "mass": np.float64, "u0": np.float64, "geom": np.float64,
                 "X": np.float64, "conn": np.int32, "elem_nn": np.int32, "bcflag": np.uint8, "dtv": np.float64,
                 "material": np.float64, "feonly": np.int32, "st_cls": np.int32, "st_nbr": np.int32,
                 "st_blk": np.float64, "tile_rows": np.int32, "tile_cls": np.int16, "lat_blk": np.float32,
                 "fe_rest": np.int32, "rel_bond": np.int32, "rel_self": np.int32, "rel_fe": np.int32,
                 "fe_adj_ptr": np.int32, "fe_adj": np.int32, "fe_conn": np.int32}


class Model:
    """A PDLSM-FEM model built from a reference command file."""

    def __init__(self, cmd_path: str, device: int = 0, precision: int = -1, lanes: int = 0, fe_lanes: int = 0,
                 verbose: int = 0):
        L = lib()
        h = _P()
        opt = Options(device, precision, lanes, verbose, fe_lanes)
        _check(L.pdx_model_create_from_cmd(cmd_path.encode(), C.byref(opt), C.byref(h)))
        self._h = h
        inf = ModelInfo()
        _check(L.pdx_model_get_info(h, C.byref(inf)))
        self.info = inf

    @classmethod
    def batch(cls, cmd_paths, device: int = 0, precision: int = -1, lanes: int = 0, fe_lanes: int = 0,
              verbose: int = 0) -> "Model":
        """Many specimens (one command file each) merged into one model (pdx_batch_create)."""
        L = lib()
        h = _P()
        opt = Options(device, precision, lanes, verbose, fe_lanes)
        arr = (C.c_char_p * len(cmd_paths))(*[p.encode() for p in cmd_paths])
        _check(L.pdx_batch_create(arr, len(cmd_paths), C.byref(opt), C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        inf = ModelInfo()
        _check(L.pdx_model_get_info(h, C.byref(inf)))
        self.info = inf
        return self

    def reaction_forces(self) -> np.ndarray:
        """Rows (U, RFx, RFy, RFz) per recorded step (RF keyword), shape (count, 4)."""
        n = C.c_int64()
        _check(lib().pdx_reaction_forces(self._h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 4))
        if n.value:
            _check(lib().pdx_reaction_forces(self._h, out.ctypes.data_as(_D), n.value, None))
        return out

    def crack_state(self) -> np.ndarray:
        """FC 1 crack rows (x0, y0, x1, y1, KI, KII, Keq, moved), shape (n_cracks, 8);
        (x1, y1) is the tip, (x0, y0) the tip before the last growth."""
        n = C.c_int()
        _check(lib().pdx_crack_state(self._h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 8))
        if n.value:
            _check(lib().pdx_crack_state(self._h, out.ctypes.data_as(_D), n.value, None))
        return out

    def crack_advance(self, tips, moved) -> None:
        """Move the cracks flagged in `moved` to `tips` (n_cracks x 2) and grow
        the PD region and break the bonds across the new segments."""
        t = np.ascontiguousarray(tips, dtype=np.float64).reshape(-1)
        mv = np.ascontiguousarray(moved, dtype=np.uint8).reshape(-1)
        _check(lib().pdx_crack_advance(self._h, t.ctypes.data_as(_D), mv.ctypes.data_as(C.POINTER(C.c_uint8))))
        self._refresh_info()

    def _refresh_info(self) -> None:
        """FC 1 growth changes the family and bond counts and the CSR size."""
        _check(lib().pdx_model_get_info(self._h, C.byref(self.info)))

    # ---- quasi-static increments ----
    def quasi_init(self) -> None:
        _check(lib().pdx_quasi_init(self._h))
        self._refresh_info()

    def quasi_step(self, method: int = 1) -> "SolveInfo":
        info = SolveInfo()
        _check(lib().pdx_quasi_step(self._h, method, C.byref(info)))
        if self.info.fail_flag == 1:
            self._refresh_info()
        return info

    # ---- implicit Newmark and the learned preconditioner ----
    def newmark_init(self) -> None:
        _check(lib().pdx_newmark_init(self._h))

    def newmark_step(self, method: int, collect: bool = False) -> "SolveInfo":
        info = SolveInfo()
        _check(lib().pdx_newmark_step(self._h, method, 1 if collect else 0, C.byref(info)))
        return info

    def learned_setup(self, cells, hidden: int = 128, seed: int = 0, max_samples: int = 4096) -> None:
        c = list(cells) + [1] * (3 - len(cells))
        _check(lib().pdx_learned_setup(self._h, c[0], c[1], c[2], hidden, seed, max_samples))

    def learned_samples(self) -> int:
        return int(lib().pdx_learned_samples(self._h))

    def learned_probe(self, nprobe: int, seed: int = 1) -> None:
        _check(lib().pdx_learned_probe(self._h, nprobe, seed))

    def learned_active(self) -> bool:
        return bool(lib().pdx_learned_active(self._h))

    def learned_options(self, trunc: int = 1, stall_window: int = 60) -> None:
        _check(lib().pdx_learned_options(self._h, trunc, stall_window))

    def learned_pairs(self):
        """(P^T r_j, coarse errors) of the collected pairs, each (count, nc) float32."""
        cnt, nc = C.c_int64(), C.c_int()
        _check(lib().pdx_learned_pairs(self._h, None, None, C.byref(cnt), C.byref(nc)))
        r = np.zeros((cnt.value, nc.value), dtype=np.float32)
        e = np.zeros_like(r)
        fp = C.POINTER(C.c_float)
        _check(lib().pdx_learned_pairs(self._h, r.ctypes.data_as(fp), e.ctypes.data_as(fp), None, None))
        return r, e

    def learned_train(self, epochs: int = 100, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_float()
        _check(lib().pdx_learned_train(self._h, epochs, lr, seed, C.byref(loss)))
        return loss.value

    def mlp_params(self, set_to: Optional[np.ndarray] = None) -> np.ndarray:
        fp = C.POINTER(C.c_float)
        n = C.c_int64()
        _check(lib().pdx_mlp_params(self._h, None, None, C.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        src = None
        if set_to is not None:
            keep = np.ascontiguousarray(set_to, dtype=np.float32)
            src = keep.ctypes.data_as(fp)
        _check(lib().pdx_mlp_params(self._h, out.ctypes.data_as(fp), src, None))
        return out

    def mlp_loss_grad(self, x: np.ndarray, t: np.ndarray, w: np.ndarray):
        fp = C.POINTER(C.c_float)
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        w = np.ascontiguousarray(w, dtype=np.float32)
        n = C.c_int64()
        _check(lib().pdx_mlp_params(self._h, None, None, C.byref(n)))
        grad = np.zeros(n.value, dtype=np.float32)
        loss = C.c_float()
        _check(lib().pdx_mlp_loss_grad(self._h, x.shape[0], x.ctypes.data_as(fp), t.ctypes.data_as(fp),
                                       w.ctypes.data_as(fp), C.byref(loss), grad.ctypes.data_as(fp)))
        return loss.value, grad

    def batch_offsets(self):
        """(node_off, member_off, eq_off), n+1 entries each, of a batched model."""
        n = lib().pdx_batch_size(self._h)
        outs = [np.zeros(n + 1, dtype=np.int64) for _ in range(3)]
        _check(lib().pdx_batch_offsets(self._h, *[o.ctypes.data_as(C.POINTER(C.c_int64)) for o in outs]))
        return tuple(outs)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pdx_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def dim(self) -> int:
        return self.info.dim

    def array(self, name: str) -> np.ndarray:
        n = C.c_int64()
        _check(lib().pdx_model_array_len(self._h, name.encode(), C.byref(n)))
        out = np.zeros(n.value, dtype=_ARRAY_DTYPES[name])
        _check(lib().pdx_model_array(self._h, name.encode(), out.ctypes.data_as(_P), n.value))
        return out

    def bond_coefficients(self):
        d = self.dim
        na = 5 if d == 2 else 9
        nd = 3 if d == 2 else 6
        A = np.zeros((self.info.n_fam, na, na))
        g = np.zeros((self.info.n_bond, d))
        dv = np.zeros((self.info.n_bond, nd))
        G = np.zeros((self.info.n_bond, d, d))
        _check(lib().pdx_bond_coefficients(self._h, _dptr(A), _dptr(g), _dptr(dv), _dptr(G)))
        return A, g, dv, G

    def internal_force(self, u_all: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_all, dtype=np.float64).reshape(-1)
        f = np.zeros(self.info.n_eq)
        _check(lib().pdx_internal_force(self._h, _dptr(u), _dptr(f)))
        return f

    def explicit_init(self) -> None:
        _check(lib().pdx_explicit_init(self._h))

    def explicit_advance(self, n: int) -> None:
        _check(lib().pdx_explicit_advance(self._h, int(n)))

    def explicit_advance_timed(self, n: int) -> float:
        ms = C.c_double()
        _check(lib().pdx_explicit_advance_timed(self._h, int(n), C.byref(ms)))
        return ms.value

    def explicit_step_host(self, u_n: np.ndarray, u_nm1: np.ndarray, out: np.ndarray) -> None:
        _check(lib().pdx_explicit_step_host(self._h, _dptr(u_n), _dptr(u_nm1), _dptr(out)))

    @property
    def steps_done(self) -> int:
        return int(lib().pdx_explicit_step_count(self._h))

    def state(self):
        N, d = self.info.n_node, self.dim
        u = np.zeros((N, d))
        sig = np.zeros((N, 6))
        phi = np.zeros(N)
        nm = int(self.array_len("fam_members"))
        bs = np.zeros(nm, dtype=np.uint8)
        _check(lib().pdx_get_state(self._h, _dptr(u), _dptr(sig), _dptr(phi), bs.ctypes.data_as(C.POINTER(C.c_uint8))))
        return u, sig, phi, bs

    def array_len(self, name: str) -> int:
        n = C.c_int64()
        _check(lib().pdx_model_array_len(self._h, name.encode(), C.byref(n)))
        return n.value

    def assemble(self, mode: int, v_all: Optional[np.ndarray] = None):
        ne, nnz = self.info.n_eq, self.info.nnz
        ia = np.zeros(ne + 1, dtype=np.int64)
        ja = np.zeros(nnz, dtype=np.int64)
        a = np.zeros(nnz)
        f = np.zeros(ne)
        v = None if v_all is None else np.ascontiguousarray(v_all, dtype=np.float64).reshape(-1)
        _check(lib().pdx_assemble_csr(self._h, int(mode), _dptr(v), ia.ctypes.data_as(C.POINTER(C.c_int64)),
                                      ja.ctypes.data_as(C.POINTER(C.c_int64)), _dptr(a), _dptr(f)))
        return ia, ja, a, f

    def run(self, results_dir: str) -> None:
        _check(lib().pdx_run(self._h, results_dir.encode()))
        self._refresh_info()


def solve_csr(ia: np.ndarray, ja: np.ndarray, a: np.ndarray, b: np.ndarray, method: int = 2,
              rtol: float = 1e-8, max_iter: int = 20000, x0: Optional[np.ndarray] = None):
    """Solve A x = b on the GPU (pdx_solve_csr).  method: 0 Jacobi PCG,
    1 block-Jacobi PCG, 2 BiCGStab (Jacobi), 3 FP32 PCG in FP64 refinement,
    6 GMRES(30) (right Jacobi), 7 FP32 BiCGStab in FP64 refinement.
    Returns (x, SolveInfo)."""
    n = len(ia) - 1
    ia = np.ascontiguousarray(ia, dtype=np.int64)
    ja = np.ascontiguousarray(ja, dtype=np.int64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    opts = SolveOpts(method, rtol, max_iter, 0 if x0 is None else 1)
    info = SolveInfo()
    code = lib().pdx_solve_csr(n, ia.ctypes.data_as(C.POINTER(C.c_int64)), ja.ctypes.data_as(C.POINTER(C.c_int64)),
                               _dptr(a), _dptr(b), _dptr(x), C.byref(opts), C.byref(info))
    if code not in (0, 7):
        _check(code)
    return x, info


def pcg_solve_noalloc(n: int, nnz: int, d_ia: int, d_ja: int, d_a: int, d_b: int, d_x: int, rtol: float = 1e-8,
                      max_iter: int = 20000, use_x0: bool = False, stream: int = 0):
    """Jacobi PCG on device arrays (raw device addresses: ia int64, ja int32,
    a, b, x float64) with the library's fixed work space; allocates nothing."""
    opts = SolveOpts(0, rtol, max_iter, 1 if use_x0 else 0)
    info = SolveInfo()
    code = lib().pdx_pcg_solve_noalloc(n, nnz, d_ia, d_ja, d_a, d_b, d_x, C.byref(opts), stream or None,
                                       C.byref(info))
    if code not in (0, 7):
        _check(code)
    return info, code
