"""ctypes mirror of ``wcfe_params`` (include/wcfe.h) and the reference constants.

The reference hard-codes every constant inside cellBP/UL_growth_explicit.cpp;
``default_params`` returns them for the three variants (kMD, k1, k31).
"""
from __future__ import annotations

import ctypes as C

LAW_LINEAR, LAW_MD_TABLE, LAW_POLY = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
VARIANT_KMD, VARIANT_K1, VARIANT_K31 = 0, 1, 2
VARIANTS = {"kMD": VARIANT_KMD, "k1": VARIANT_K1, "k31": VARIANT_K31}


class Params(C.Structure):
    _fields_ = [
        ("mu", C.c_double), ("thick", C.c_double), ("thetag_dot", C.c_double), ("kappa", C.c_double),
        ("tact_rate", C.c_double), ("tact_t1", C.c_double), ("tact_max", C.c_double),
        ("D_A", C.c_double), ("D_C", C.c_double),
        ("force_law", C.c_int32), ("linear_norm2d", C.c_int32),
        ("k_lin", C.c_double), ("rest_len", C.c_double), ("poly_k0", C.c_double), ("poly_x0", C.c_double),
        ("rho_i_max", C.c_double),
        ("k_on", C.c_double), ("ka", C.c_double), ("kb", C.c_double), ("Fa", C.c_double), ("Fb", C.c_double),
        ("k_bend", C.c_double), ("k_area", C.c_double), ("area0", C.c_double),
        ("ap_rate", C.c_double), ("ap_force", C.c_double), ("ap_density", C.c_double),
        ("ap_enable", C.c_int32), ("seed", C.c_uint32), ("stream", C.c_uint32),
        ("drag", C.c_double), ("damp", C.c_double), ("rho", C.c_double),
        ("protrude_v", C.c_double), ("protrude_cx", C.c_double), ("protrude_cy", C.c_double),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p


def default_params(variant: str | int = "kMD") -> Params:
    """Reference constants (UL_growth_explicit.cpp) for one integrin variant."""
    v = VARIANTS[variant] if isinstance(variant, str) else int(variant)
    p = Params()
    p.mu, p.thick, p.thetag_dot, p.kappa = 1000.0, 1.0, 0.0, 0.5
    p.tact_rate, p.tact_t1, p.tact_max = 200.0, 2.0, 400.0
    p.D_A, p.D_C = 1.0, 1e-10
    if v == VARIANT_KMD:
        p.force_law, p.k_lin, p.linear_norm2d = LAW_MD_TABLE, 31000.0, 0
    elif v == VARIANT_K1:
        p.force_law, p.k_lin, p.linear_norm2d = LAW_LINEAR, 1000.0, 1
    else:
        p.force_law, p.k_lin, p.linear_norm2d = LAW_LINEAR, 31000.0, 1
    p.rest_len, p.poly_k0, p.poly_x0 = 0.0, 31000.0, 0.005
    p.rho_i_max = 100.0
    p.k_on, p.ka, p.kb, p.Fa, p.Fb = 1.0, 0.004, 10.0, 15.0, 15.0
    p.k_bend, p.k_area, p.area0 = 20.0, 1.0, 10 * 10 * 3.1416
    p.ap_rate, p.ap_force, p.ap_density, p.ap_enable = 10.0, 5.0, 100.0, 1
    p.seed, p.stream = 1, 0
    p.drag, p.damp, p.rho = 0.001, 0.001, 1.0
    return p


def kint_for(variant: str) -> float:
    """The kint cellBP/main.cpp passes to updateFA for each variant (kMD: -1, unused)."""
    return {"kMD": -1.0, "k1": 1000.0, "k31": 31000.0}[variant]
