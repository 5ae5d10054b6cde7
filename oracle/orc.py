"""ctypes binding of the CPU oracle (oracle/pdx_oracle.c).

Test infrastructure: used only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker of the CUDA path.  The oracle is
built from the host-setup arrays of a model (pdx.Model(..., device=-1) gives
them without a GPU).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "pdx_oracle.c")
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "pdx_oracle.h"))):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", src, "-o", LIB_PATH, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


class OrcModel(C.Structure):
    _fields_ = [("dim", C.c_int), ("protype", C.c_int), ("n_node", C.c_int), ("n_elem", C.c_int),
                ("n_eq", C.c_int), ("n_fam", C.c_int), ("n_pdbe", C.c_int), ("n_fe", C.c_int),
                ("X", C.c_void_p), ("conn", C.c_void_p), ("elem_nn", C.c_void_p), ("fe_idx", C.c_void_p),
                ("eq", C.c_void_p), ("vol_node", C.c_void_p), ("vol_elem", C.c_void_p), ("fam_off", C.c_void_p),
                ("fam_members", C.c_void_p), ("fam_delta", C.c_void_p), ("fam_cdv", C.c_void_p),
                ("pdbe", C.c_void_p), ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("nlf", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcModel), C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_coeffs.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_internal_force.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_lumped_mass.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_explicit.restype = C.c_int64
        L.orc_explicit.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                   C.c_uint64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_stress.argtypes = [C.c_void_p] * 5
        L.orc_assemble.argtypes = [C.c_void_p] * 7
        L.orc_consistent_mass.argtypes = [C.c_void_p] * 4
        L.orc_bond_uniform.restype = C.c_double
        L.orc_bond_uniform.argtypes = [C.c_uint64, C.c_int, C.c_int]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class Oracle:
    """Oracle context for the model whose host arrays ``model`` (a pdx.Model) exposes."""

    def __init__(self, model, nthreads: int = 0):
        a = {}
        for name in ("X", "conn", "elem_nn", "fe_idx", "eq", "vol_node", "vol_elem", "fam_off", "fam_members",
                     "fam_horizon", "fam_cdv", "pdbe", "bond_state0", "u0", "bcflag", "dtv", "material",
                     "csr_ia", "csr_ja"):
            a[name] = np.ascontiguousarray(model.array(name))
        self.a = a
        info = model.info
        mat = a["material"]
        self.dim = info.dim
        self.n_node = info.n_node
        self.n_eq = info.n_eq
        self.dt = float(mat[8])
        self.nsteps = int(mat[9])
        self.s0 = float(mat[10])
        self.seed = int(mat[11])
        self.pert = float(mat[12])
        self.m = OrcModel(info.dim, int(mat[7]), info.n_node, info.n_elem, info.n_eq, info.n_fam, info.n_pdbe,
                          info.n_fe, _p(a["X"]), _p(a["conn"]), _p(a["elem_nn"]), _p(a["fe_idx"]), _p(a["eq"]),
                          _p(a["vol_node"]), _p(a["vol_elem"]), _p(a["fam_off"]), _p(a["fam_members"]),
                          _p(a["fam_horizon"]), _p(a["fam_cdv"]), _p(a["pdbe"]), float(mat[0]), float(mat[1]),
                          float(mat[2]), float(mat[5]))
        self.h = lib().orc_create(C.byref(self.m), int(nthreads))
        if not self.h:
            raise RuntimeError("oracle: singular moment matrix")
        self.bond_state = a["bond_state0"].copy()
        self.n_fam = info.n_fam
        self.n_bond = info.n_bond

    def close(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def coeffs(self):
        d = self.dim
        na, nd = (5, 3) if d == 2 else (9, 6)
        A = np.zeros((self.n_fam, na, na)); g = np.zeros((self.n_bond, d))
        dv = np.zeros((self.n_bond, nd)); G = np.zeros((self.n_bond, d, d))
        lib().orc_coeffs(self.h, _p(A), _p(g), _p(dv), _p(G))
        return A, g, dv, G

    def internal_force(self, u_all: np.ndarray, bond_state: Optional[np.ndarray] = None) -> np.ndarray:
        bs = self.bond_state if bond_state is None else np.ascontiguousarray(bond_state, dtype=np.uint8)
        u = np.ascontiguousarray(u_all, dtype=np.float64).reshape(-1)
        f = np.zeros(self.n_eq)
        lib().orc_internal_force(self.h, _p(bs), _p(u), _p(f))
        return f

    def lumped_mass(self) -> np.ndarray:
        m = np.zeros(self.n_eq)
        lib().orc_lumped_mass(self.h, _p(m))
        return m

    def explicit(self, nsteps: Optional[int] = None, dt: Optional[float] = None, s0: Optional[float] = None,
                 keep_traj: bool = False, u0: Optional[np.ndarray] = None):
        """Run the explicit solver from the model's initial state; returns (u, bond_state, traj, nbroken)."""
        n = self.nsteps if nsteps is None else nsteps
        dt_ = self.dt if dt is None else dt
        s0_ = self.s0 if s0 is None else s0
        u = np.ascontiguousarray(self.a["u0"] if u0 is None else u0, dtype=np.float64).copy()
        bs = self.a["bond_state0"].copy()
        traj = np.zeros((n + 1, self.n_node * self.dim)) if keep_traj else None
        nb = lib().orc_explicit(self.h, dt_, n, _p(self.a["bcflag"]), _p(self.a["dtv"]), s0_, self.seed,
                                self.pert, _p(u), _p(bs), _p(traj))
        self.bond_state = bs
        return u.reshape(self.n_node, self.dim), bs, traj, nb

    def stress(self, u_all: np.ndarray, bond_state: Optional[np.ndarray] = None):
        bs = self.bond_state if bond_state is None else np.ascontiguousarray(bond_state, dtype=np.uint8)
        u = np.ascontiguousarray(u_all, dtype=np.float64).reshape(-1)
        sig = np.zeros((self.n_node, 6)); phi = np.zeros(self.n_node)
        lib().orc_stress(self.h, _p(bs), _p(u), _p(sig), _p(phi))
        return sig, phi

    def assemble(self, v_all: np.ndarray, bond_state: Optional[np.ndarray] = None):
        bs = self.bond_state if bond_state is None else np.ascontiguousarray(bond_state, dtype=np.uint8)
        ia, ja = self.a["csr_ia"], self.a["csr_ja"]
        a = np.zeros(len(ja)); f = np.zeros(self.n_eq)
        v = np.ascontiguousarray(v_all, dtype=np.float64).reshape(-1)
        lib().orc_assemble(self.h, _p(bs), _p(ia), _p(ja), _p(v), _p(a), _p(f))
        return ia, ja, a, f

    def consistent_mass(self):
        ia, ja = self.a["csr_ia"], self.a["csr_ja"]
        a = np.zeros(len(ja))
        lib().orc_consistent_mass(self.h, _p(ia), _p(ja), _p(a))
        return a
