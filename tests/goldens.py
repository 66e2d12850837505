"""Loaders for the golden fixtures in tests/golden (made by make_golden.py from
the reference's own source) and the matching oracle parameter sets."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SP_CASES = ["sp_cavity8", "sp_poiseuille", "sp_pressure", "sp_mixed"]
TP_CASES = ["tp_drain", "tp_periodic", "tp_velbc"]
GREY_CASES = ["grey_channel", "grey_mixed", "grey_faces"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def params_of(d):
    return json.loads(str(d["params"]))


def oracle_params(d, ref_emulation=0):
    from oracle.oracle import make_params
    P = params_of(d)
    shape = tuple(int(x) for x in d["shape"])
    if str(d["kind"]) == "single_phase_class":
        return make_params(shape, niu=P["niu"], force=(P["fx"], P["fy"], P["fz"]), bc=P["bc"],
                           rho_bc=P["rho_bc"], vel_bc=P["vel_bc"])
    if str(d["kind"]) == "grey_script":
        return make_params(shape, niu=P["niu"], force=P["force"], bc=P["bc"], rho_bc=P["rho_bc"],
                           vel_bc=P["vel_bc"], visc_convention=1, guo_convention=1, bc_form=1, grey=True)
    return make_params(shape, force=P["force"], bc=P["bc"], rho_bc=P["rho_bc"], vel_bc=P["vel_bc"],
                       visc_convention=1, guo_convention=1, bc_form=1, two_phase=True,
                       niu_l=P["niu_l"], niu_g=P["niu_g"], psi_solid=P["psi_solid"], cap_a=P["CapA"],
                       psi_bc=P["psi_bc"], psi_val=P["psi_val"], ref_emulation=ref_emulation)


def cavity_solid_50():
    d = load("sp_cavity50")
    bits = np.unpackbits(d["solid_bits"])[: 50 * 50 * 50]
    return bits.reshape((50, 50, 50), order="F").astype(np.int8)


def normwise_rel(a, b, mask):
    """max|a-b| / max|b| over the cells in mask (all components)."""
    den = np.abs(b[mask]).max()
    return float(np.abs(a[mask] - b[mask]).max() / (den if den > 0 else 1.0))


def grey_solid(ns):
    """solid = ns.astype(int) != 0 (Grey_Scale/lbm_solver_3d_Macro_Sukop.py:321)."""
    return (np.asarray(ns).astype(int) != 0).astype(np.int8)
