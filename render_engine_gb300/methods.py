"""Cache methods and the method tables of each command-line mode.

A method is the reference's ``Method`` record (cuda/poc_gpu.cu:803-805): how many rays a
cache point traces per frame, how long its history is, whether dependencies are tracked,
and what happens on a light or geometry event.  The tables below list, for every mode of
the command line, the methods that mode runs, in the reference's order and with the
reference's display names, so that JSONL consumers see the same rows:

* ``timing``  -- cuda/poc_gpu.cu:1348-1358
* ``res``     -- cuda/poc_gpu.cu:1326-1330
* ``scen``    -- cuda/poc_gpu.cu:1451-1469
* ``scenf``   -- cuda/poc_gpu.cu:1404-1418 (responsive mask and budgets depend on the scene)
* ``quality`` -- cuda/poc_gpu.cu:1019-1045
* ``recon``   -- cuda/poc_gpu.cu:1493-1497
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field, fields


@dataclass
class Method:
    name: str
    mode: int
    nmax: float
    budget: float
    deps: bool = False
    verify: bool = False
    oracle: bool = False
    track_every: int = 1
    rescale: bool = False
    resp_mask: int = 0
    nmax_resp: float = 8.0
    ddgi: bool = False
    ddgi_h: float = 0.97
    ddgi_thr: float = 0.25
    ddgi_clamp: bool = True
    memory: bool = False
    ramp: bool = False
    wake_verify: bool = False
    snaps: bool = False
    proj: bool = False
    snap_verify: bool = False
    rays: float = 1.0

    def replace(self, **kw) -> "Method":
        d = {f.name: getattr(self, f.name) for f in fields(self)}
        d.update(kw)
        return Method(**d)


class CMethod(ctypes.Structure):
    """C layout shared by ``rc_method`` (include/rc_api.h) and the CPU oracle's ``osc_method``."""
    _fields_ = [
        ("mode", ctypes.c_int), ("nmax", ctypes.c_float), ("budget", ctypes.c_float),
        ("deps", ctypes.c_int), ("verify", ctypes.c_int), ("oracle", ctypes.c_int),
        ("track_every", ctypes.c_int), ("rescale", ctypes.c_int), ("resp_mask", ctypes.c_int),
        ("nmax_resp", ctypes.c_float), ("ddgi", ctypes.c_int), ("ddgi_h", ctypes.c_float),
        ("ddgi_thr", ctypes.c_float), ("ddgi_clamp", ctypes.c_int), ("memory", ctypes.c_int),
        ("ramp", ctypes.c_int), ("wake_verify", ctypes.c_int), ("snaps", ctypes.c_int),
        ("proj", ctypes.c_int), ("snap_verify", ctypes.c_int), ("rays", ctypes.c_float),
    ]


def to_c(m: Method) -> CMethod:
    c = CMethod()
    for name, ctype in CMethod._fields_:
        v = getattr(m, name)
        setattr(c, name, int(v) if ctype is ctypes.c_int else float(v))
    return c


def _m(name, mode, nmax, budget, deps=False, verify=False, oracle=False, track_every=1, **kw) -> Method:
    return Method(name, mode, float(nmax), float(budget), deps, verify, oracle, track_every, **kw)


def timing_methods() -> list[Method]:
    return [
        _m("Classique 1.0x", 0, 16, 1.0),
        _m("Classique 2.0x", 0, 16, 2.0),
        _m("SHaRC responsive 1.0x", 0, 32, 1.0, resp_mask=1, rescale=True),
        _m("DDGI 1.0x", 0, 64, 1.0, ddgi=True, rescale=True),
        _m("v3 sans suivi", 1, 64, 1.0, False, True, False),
        _m("v3 complet", 1, 64, 1.0, True, True, False, 1),
        _m("v3 suivi 1 frame sur 2", 1, 64, 1.0, True, True, False, 2),
        _m("v3 suivi 1 frame sur 4", 1, 64, 1.0, True, True, False, 4),
        _m("v4-A2C suivi 1/4", 1, 64, 1.0, True, True, False, 4, memory=True, wake_verify=True, ramp=True),
    ]


def res_methods() -> list[Method]:
    return [
        _m("Classique", 0, 16, 1.0),
        _m("SHaRC responsive", 0, 64, 1.0, resp_mask=1, rescale=True),
        _m("v3", 1, 64, 1.0, True, True, False, 4),
        _m("v4-A2C", 1, 64, 1.0, True, True, False, 4, memory=True, wake_verify=True, ramp=True),
    ]


def scen_methods() -> list[Method]:
    S = dict(resp_mask=1, nmax_resp=8.0, rescale=True)
    v4 = dict(deps=True, verify=True, track_every=4)
    return [
        _m("SHaRC N=64 resp=8, 1.57x", 0, 64, 1.57, **S),
        _m("Accumulation+parlampe N=32, 1.53x", 0, 32, 1.53, rescale=True),
        _m("SHaRC + memoire naive, 1.57x", 0, 64, 1.57, memory=True, **S),
        _m("Accum+parlampe + memoire naive N=32, 1.53x", 0, 32, 1.53, rescale=True, memory=True),
        _m("Accum+parlampe + memoire naive N=64, 1.53x", 0, 64, 1.53, rescale=True, memory=True),
        _m("SHaRC + memoire + instantanes, 1.57x", 0, 64, 1.57, memory=True, snaps=True, **S),
        _m("Accum + memoire + instantanes N=32, 1.53x", 0, 32, 1.53, rescale=True, memory=True, snaps=True),
        _m("Accum + memoire + instantanes N=64, 1.53x", 0, 64, 1.53, rescale=True, memory=True, snaps=True),
        _m("Oracle", 1, 64, 1.0, oracle=True),
        _m("v3", 1, 64, 1.0, **v4),
        _m("v4-A memoire", 1, 64, 1.0, memory=True, **v4),
        _m("v4-C rampe", 1, 64, 1.0, ramp=True, **v4),
        _m("v4-AC memoire+rampe", 1, 64, 1.0, memory=True, ramp=True, **v4),
        _m("v4-A2 memoire verifiee", 1, 64, 1.0, memory=True, wake_verify=True, **v4),
        _m("v4-A2C memoire verifiee+rampe", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, **v4),
        _m("v5-A instantanes verifies", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, snap_verify=True, **v4),
        _m("v5-A instantanes", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, **v4),
        _m("v5-AB instantanes+projection", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, proj=True, **v4),
    ]


SCEN_SCENARIOS = [
    ("R1 allumee-eteinte-rallumee", [(0, 50), (1, 30), (0, 50)]),
    ("R2 allumee-eteinte-porte-rallumee", [(0, 40), (1, 20), (2, 20), (3, 50)]),
    ("R3 porte ouverte-fermee-rouverte", [(0, 50), (3, 30), (0, 50)]),
    ("I1 lampe eteinte", [(0, 50), (1, 50)]),
    ("I2 porte", [(1, 50), (2, 50)]),
    ("I3 lampe allumee 1re fois", [(2, 50), (3, 50)]),
    ("I4 boite", [(3, 50), (4, 50)]),
]


def scenf_methods(dyn_mask: int, bS: float = 1.57, bA: float = 1.53) -> list[Method]:
    """Methods of ``scenf``; ``dyn_mask`` = lights whose intensity differs from state 0."""
    S = dict(resp_mask=dyn_mask, nmax_resp=8.0, rescale=True)
    v4 = dict(deps=True, verify=True, track_every=4)
    return [
        _m("SHaRC N=64 resp=8, %.2fx" % bS, 0, 64, bS, **S),
        _m("SHaRC + memoire naive, %.2fx" % bS, 0, 64, bS, memory=True, **S),
        _m("Accumulation+parlampe N=32, %.2fx" % bA, 0, 32, bA, rescale=True),
        _m("Accum+parlampe + memoire naive N=32, %.2fx" % bA, 0, 32, bA, rescale=True, memory=True),
        _m("Accum+parlampe + memoire naive N=64, %.2fx" % bA, 0, 64, bA, rescale=True, memory=True),
        _m("SHaRC + memoire + instantanes, %.2fx" % bS, 0, 64, bS, memory=True, snaps=True, **S),
        _m("Accum + memoire + instantanes N=32, %.2fx" % bA, 0, 32, bA, rescale=True, memory=True, snaps=True),
        _m("Accum + memoire + instantanes N=64, %.2fx" % bA, 0, 64, bA, rescale=True, memory=True, snaps=True),
        _m("Oracle", 1, 64, 1.0, oracle=True),
        _m("v3", 1, 64, 1.0, **v4),
        _m("v4-A2C memoire verifiee+rampe", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, **v4),
        _m("v5-A instantanes verifies", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, snap_verify=True, **v4),
        _m("v5-A instantanes", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, **v4),
        _m("v5-AB instantanes+projection", 1, 64, 1.0, memory=True, wake_verify=True, ramp=True, snaps=True, proj=True, **v4),
    ]


def quality_methods(budgets: list[float]) -> list[Method]:
    out = []
    for b in budgets:
        for N in (8, 16, 32):
            out.append(_m("Accumulation N=%d, %.2fx rayons" % (N, b), 0, N, b))
            out.append(_m("Accumulation+parlampe N=%d, %.2fx rayons" % (N, b), 0, N, b, rescale=True))
        for N in (16, 32, 64):
            for R in (4, 8):
                out.append(_m("SHaRC N=%d resp=%d, %.2fx rayons" % (N, R, b), 0, N, b, resp_mask=1, nmax_resp=float(R), rescale=True))
        for h in (0.9, 0.97):
            for t in (0.25, 0.5, 1.0):
                for cl in (0, 1):
                    for pl in (0, 1):
                        out.append(_m("DDGI%s h=%.2f seuil=%.2f borne=%d, %.2fx rayons" % ("+parlampe" if pl else "", h, t, cl, b),
                                      0, 64, b, ddgi=True, ddgi_h=h, ddgi_thr=t, ddgi_clamp=bool(cl), rescale=bool(pl)))
    out.append(_m("Cache a dependances v3", 1, 64, 1.0, True, True, False, 1))
    out.append(_m("Cache a dependances v3, suivi 1/4", 1, 64, 1.0, True, True, False, 4))
    out.append(_m("Oracle", 1, 64, 1.0, oracle=True))
    return out


def recon_methods() -> list[Method]:
    return [
        _m("Cache a dependances v3, suivi 1/4", 1, 64, 1.0, True, True, False, 4),
        _m("SHaRC N=64 resp=8, 1.52x", 0, 64, 1.52, resp_mask=1, nmax_resp=8.0, rescale=True),
        _m("Accumulation+parlampe N=32, 1.51x", 0, 32, 1.51, rescale=True),
        _m("Oracle", 1, 64, 1.0, oracle=True),
    ]


def by_name(table: list[Method], name: str) -> Method:
    for m in table:
        if m.name == name:
            return m
    raise KeyError(name)


def sequence(parts: list[tuple[int, int]]) -> list[int]:
    seq: list[int] = []
    for state, frames in parts:
        seq += [state] * frames
    return seq
