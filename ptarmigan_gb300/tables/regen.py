"""Regenerates the reference tables that are missing from its source tree.

``nonlinear_compton/cp/tables/cdf.rs`` (the CP harmonic CDF) is absent from
the reference; this runs its generator on the GPU
(``ptg_regen_nlc_cp_cdf``) and writes ``nlc_cp_cdf.ptgt`` plus the total
rates it computed (``nlc_cp_cdf_totals.ptgt``), which must reproduce the
shipped total-rate table ``nlc_cp_rate.ptgt``.

``pair_creation/lp/tables/mid_range/cdf.rs`` (the LP Breit-Wheeler
mid-range CDF) is absent as well: ``ptg_regen_bw_lp_mid_cdf`` runs its
generator and writes ``bw_lp_mid_cdf.ptgt``; its totals must reproduce the
shipped ``bw_lp_mid_total.ptgt``.

    python ptarmigan_gb300/tables/regen.py --out DIR [--which cp,lpm]
"""

import argparse
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ptarmigan_gb300 import build, engine  # noqa: E402
from ptarmigan_gb300.tables.extract import read_ptgt, write_ptgt  # noqa: E402


def regen_cp(out_dir):
    build.build()
    L = engine.load()
    L.ptg_regen_nlc_cp_cdf.restype = C.c_int
    L.ptg_regen_nlc_cp_cdf.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    eng = engine.Engine()
    cdf = np.zeros(4270 * 64)
    tot = np.zeros(4270)
    st = L.ptg_regen_nlc_cp_cdf(eng._h, cdf.ctypes.data_as(C.POINTER(C.c_double)),
                                 tot.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise RuntimeError(L.ptg_last_error().decode())
    eng.close()
    write_ptgt(os.path.join(out_dir, "nlc_cp_cdf.ptgt"), (4270, 32, 2), cdf.tolist())
    write_ptgt(os.path.join(out_dir, "nlc_cp_cdf_totals.ptgt"), (70, 61), tot.tolist())
    _, shipped = read_ptgt(os.path.join(HERE, "data", "nlc_cp_rate.ptgt"))
    shipped = np.exp(np.array(shipped))
    rel = np.abs(tot - shipped) / shipped
    print("CP CDF regenerated: max |total - shipped| / shipped = %.3e (median %.3e)" % (rel.max(), np.median(rel)))
    return rel


def regen_lp_mid(out_dir):
    build.build()
    L = engine.load()
    L.ptg_regen_bw_lp_mid_cdf.restype = C.c_int
    L.ptg_regen_bw_lp_mid_cdf.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    eng = engine.Engine()
    cdf = np.zeros(5652 * 48)
    tot = np.zeros(5652 * 2)
    st = L.ptg_regen_bw_lp_mid_cdf(eng._h, cdf.ctypes.data_as(C.POINTER(C.c_double)),
                                    tot.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise RuntimeError(L.ptg_last_error().decode())
    eng.close()
    write_ptgt(os.path.join(out_dir, "bw_lp_mid_cdf.ptgt"), (5652, 16, 3), cdf.tolist())
    _, shipped = read_ptgt(os.path.join(HERE, "data", "bw_lp_mid_total.ptgt"))
    shipped = np.exp(np.array(shipped))
    ok = shipped > 0.0
    rel = np.abs(tot[ok] - shipped[ok]) / shipped[ok]
    zero_ok = np.all(tot[~ok] == 0.0)
    print("LP BW mid-range CDF regenerated: max |total - shipped| / shipped = %.3e (median %.3e), "
          "zero totals reproduced: %s" % (rel.max(), np.median(rel), zero_ok))
    return rel


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "data"))
    ap.add_argument("--which", default="cp,lpm")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    which = args.which.split(",")
    if "cp" in which:
        regen_cp(args.out)
    if "lpm" in which:
        regen_lp_mid(args.out)
