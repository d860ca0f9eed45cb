"""The reference's own PD-IPC kernels, run on the host (test infrastructure).

oracle/build_ref.py compiles Simulator/PD-IPC/PdIpcGpuFunc.cu of the reference
with oracle/cuda_emu.h into oracle/_ref/libpdipc_ref_{fp32,fp64}.so;
oracle/ref_harness.cpp exposes its kernels in the reference's host order.
This module feeds them the oracle's initialised tables, converted to the
reference's layouts (PdIpcSimulator::gpuSolverInit, PdIpcSimulator.cpp:563-882),
so the oracle's restatement can be checked against the reference's own
arithmetic on the same inputs.  Only tests/golden/make_ref_fixtures.py runs
it: the reference tree is needed to build it, and the fixtures it writes are
what the tests read.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref

_libs: dict[str, C.CDLL] = {}


def available() -> bool:
    return build_ref.reference_dir() is not None


def _lib(variant: str) -> C.CDLL:
    if variant not in _libs:
        paths = build_ref.build()
        if paths is None:
            raise RuntimeError("the reference tree is not here: set PDIPC_REFERENCE_DIR")
        _libs[variant] = C.CDLL(paths[variant])
    return _libs[variant]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefKernels:
    """One build of the reference kernels (qeal = float32 or float64)."""

    def __init__(self, variant: str = "fp32"):
        self.L = _lib(variant)
        self.dt = np.float32 if variant == "fp32" else np.float64
        self.L.ref_qeal_bytes.restype = C.c_int
        assert self.L.ref_qeal_bytes() == np.dtype(self.dt).itemsize
        q = C.c_float if variant == "fp32" else C.c_double
        self.q = q
        vp = C.c_void_p
        self.L.ref_predict.argtypes = [C.c_int, q] + [vp] * 9
        self.L.ref_local_projection.argtypes = [C.c_int] + [vp] * 11 + [C.c_int] + [vp] * 4
        self.L.ref_update_operators.argtypes = [C.c_int, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, C.c_int] + [vp] * 5
        self.L.ref_chebyshev_r2.argtypes = [C.c_int, C.c_int] + [vp] * 14
        self.L.ref_toi_per_candidate.argtypes = [C.c_int, vp, vp, vp, vp]
        self.L.ref_toi_global.argtypes = [C.c_int, vp, vp, vp, vp]
        self.L.ref_toi_global.restype = q
        self.L.ref_contact.argtypes = [q, q, q, C.c_int, vp, vp, vp, vp, vp, C.c_int]

    def a(self, x):
        return np.ascontiguousarray(x, dtype=self.dt)

    # ------------------------------------------------------------------ tables
    def tables(self, orc):
        """Reference-layout tables from an oracle built in the R2-operator form."""
        t = {k: orc.table(k) for k in ("lOff", "lNum", "lNbr", "lStrain", "lRest", "lLbo", "lBend", "curvNorm",
                                      "invMass", "grav", "pinFlag", "pinStiff", "Delastic", "nPtr", "nCol", "nVal",
                                      "r2Ptr", "r2Col", "r2Const", "r2First", "pathPtr", "pathK", "pathA", "collMass",
                                      "Xrest")}
        n = len(t["lOff"])
        r = {"n": n, "ntot": len(t["collMass"])}
        i32 = lambda x: np.ascontiguousarray(x, dtype=np.int32)  # noqa: E731
        for k in ("lOff", "lNum", "lNbr", "pinFlag"):
            r[k] = i32(t[k])
        for k in ("lStrain", "lRest", "lLbo", "lBend", "curvNorm", "invMass", "grav", "Delastic", "collMass", "Xrest"):
            r[k] = self.a(t[k])
        pins = np.nonzero(t["pinFlag"] >= 0)[0]
        r["pinIndex"] = i32(pins)
        r["pinStiff"] = self.a(t["pinStiff"][t["pinFlag"][pins]]) if pins.size else self.a(np.zeros(1))
        # R1 rows: [self (value 0), off-diagonals ascending] (PdIpcSimulator.cpp:640-672)
        nPtr, nCol, nVal = t["nPtr"], t["nCol"], t["nVal"]
        r1Index, r1Value, r1Dii, r1Num, r1Off = [], [], [], [], []
        off = 0
        for i in range(n):
            cols = nCol[nPtr[i]:nPtr[i + 1]]
            r1Index += [i] + cols.tolist()
            r1Value += [0.0] + nVal[nPtr[i]:nPtr[i + 1]].tolist()
            r1Dii += [i] * (1 + len(cols))
            r1Num.append(1 + len(cols))
            r1Off.append(off)
            off += 1 + len(cols)
        r.update(r1Index=i32(r1Index), r1Value=self.a(r1Value), r1Dii=i32(r1Dii), r1Num=i32(r1Num),
                 r1Off=i32(r1Off))
        # R2 rows, their path terms and first-order slots (cpp:700-882)
        r2Ptr, pathPtr = t["r2Ptr"], t["pathPtr"]
        nR2 = len(t["r2Col"])
        rowOf = np.repeat(np.arange(n), np.diff(r2Ptr))
        first = t["r2First"].astype(np.int64)
        mapped = np.where(first >= 0, first - nPtr[rowOf] + 1 + np.asarray(r1Off)[rowOf], -1)
        r.update(r2Index=i32(t["r2Col"]), r2Num=i32(np.diff(r2Ptr)), r2Off=i32(r2Ptr[:-1]),
                 r2Const=self.a(t["r2Const"]), r2First=i32(mapped),
                 r2RowNum=i32(np.diff(pathPtr)), r2RowOff=i32(pathPtr[:-1]),
                 aijk=self.a(t["pathA"]), r2Djj=i32(t["pathK"]),
                 r2Dii=i32(np.repeat(rowOf, np.diff(pathPtr))))
        assert len(r["r2RowNum"]) == nR2
        return r

    # ------------------------------------------------------------------ stages
    def pd_stage(self, T, X, V, dt, lg=10, cheby=15):
        """advance's prediction and one outer iteration's solve without contact
        (PdIpcSimulator.cpp:1683-1711 then LocalGlobalIteration cpp:1554-1622):
        positions after `lg` local-global iterations, from positions X (all
        points, 3 x ntot) and velocities V (3 x n)."""
        n, ntot = T["n"], T["ntot"]
        pts = self.a(np.asarray(X, np.float64).reshape(-1)).copy()
        vel = self.a(np.asarray(V, np.float64).reshape(-1)).copy()
        initRhs = np.zeros(3 * n, self.dt)
        inert = np.zeros(n, self.dt)
        zeros3 = np.zeros(3 * n, self.dt)
        self.L.ref_predict(n, self.q(dt), _p(pts), _p(vel), _p(initRhs), _p(inert), _p(T["grav"]), _p(zeros3),
                           _p(np.zeros(3 * ntot, self.dt)), _p(T["invMass"]), _p(T["pinFlag"]))
        # sysDiag = elastic + inertial (the cudaMemcpy and cublasSaxpy of cpp:1557-1558)
        sysDiag = (T["Delastic"] + inert).astype(self.dt)
        r1Ops = np.zeros(len(T["r1Value"]), self.dt)
        r2PathOps = np.zeros(len(T["aijk"]), self.dt)
        r2RowOps = np.zeros(len(T["r2Index"]), self.dt)
        self.L.ref_update_operators(len(T["r1Value"]), _p(sysDiag), _p(T["r1Value"]), _p(T["r1Dii"]), _p(r1Ops),
                                    len(T["aijk"]), _p(T["aijk"]), _p(T["r2Dii"]), _p(T["r2Djj"]), _p(r2PathOps),
                                    len(T["r2Index"]), _p(T["r2RowNum"]), _p(T["r2RowOff"]), _p(T["r2Const"]),
                                    _p(T["r2First"]), _p(r2RowOps))
        rhs = np.zeros(3 * n, self.dt)
        first = np.zeros(3 * n, self.dt)
        pre = np.zeros(3 * n, self.dt)
        nxt = np.zeros(3 * n, self.dt)
        restPts = self.a(T["Xrest"]).copy()
        for _ in range(lg):
            self.L.ref_local_projection(n, _p(initRhs), _p(T["lStrain"]), _p(T["lBend"]), _p(T["lNbr"]),
                                        _p(T["lNum"]), _p(T["lOff"]), _p(T["lRest"]), _p(T["lLbo"]),
                                        _p(T["curvNorm"]), _p(pts), None, len(T["pinIndex"]), _p(restPts),
                                        _p(T["pinIndex"]), _p(T["pinStiff"]), _p(rhs))
            self.L.ref_chebyshev_r2(cheby, n, _p(sysDiag), _p(rhs), _p(r1Ops), _p(T["r1Index"]), _p(T["r1Num"]),
                                    _p(T["r1Off"]), _p(first), _p(pre), _p(pts), _p(nxt), _p(r2RowOps),
                                    _p(T["r2Index"]), _p(T["r2Num"]), _p(T["r2Off"]))
        return pts.reshape(-1, 3).astype(np.float64)

    @staticmethod
    def candidate_list(pt, ee):
        """The reference's 5-int candidate records [type, v0..v3] (type 0
        point-triangle, 1 edge-edge), point-triangle ones first."""
        pt = np.asarray(pt, np.int32).reshape(-1, 4)
        ee = np.asarray(ee, np.int32).reshape(-1, 4)
        lst = np.concatenate([np.column_stack([np.zeros(len(pt), np.int32), pt]),
                              np.column_stack([np.ones(len(ee), np.int32), ee])])
        return np.ascontiguousarray(lst, dtype=np.int32)

    def toi(self, lst, x0, x1):
        """(per-candidate toi, global clamped toi) of getImpactOfTimeKernel."""
        n = len(lst)
        a0 = self.a(np.asarray(x0).reshape(-1))
        a1 = self.a(np.asarray(x1).reshape(-1))
        per = np.ones(max(n, 1), self.dt)
        self.L.ref_toi_per_candidate(n, _p(lst), _p(a0), _p(a1), _p(per))
        blocks = np.ones(max((n + 511) // 512, 1), self.dt)
        g = self.L.ref_toi_global(n, _p(lst), _p(a0), _p(a1), _p(blocks))
        return per[:n].astype(np.float64), float(g)

    def contact(self, lst, x, mass, dhat, kappa, dt):
        """(collision diagonal, collision rhs) of setCollisionConstraintsKernel."""
        ntot = len(mass)
        ax = self.a(np.asarray(x).reshape(-1))
        diag = np.zeros(ntot, self.dt)
        rhs = np.zeros(3 * ntot, self.dt)
        self.L.ref_contact(self.q(dhat), self.q(kappa), self.q(dt), len(lst), _p(lst), _p(ax), _p(self.a(mass)),
                           _p(diag), _p(rhs), ntot)
        return diag.astype(np.float64), rhs.reshape(-1, 3).astype(np.float64)
