"""Extract the reference's numeric physics tables into files this package can load.

Ptarmigan stores every precomputed rate, CDF and quadrature rule as a Rust
numeric literal (``static NAME: [[f64; 2]; 41] = [...]``).  The tables are
data that the physics depends on, so they have to be the same numbers here.
This script reads those literals from a ptarmigan source tree and writes:

* ``ptg_tables_small.h`` — the small tables (< 64 KB each) and the scalar
  grid constants as C arrays.  The includer picks the storage class through
  ``PTG_TABLE_DECL`` (``static const`` on the host, ``static __device__ const``
  in CUDA), so the same header serves the oracle and the kernels.
* ``data/*.ptgt`` — the large LMA tables as a tiny binary format:
  ``b"PTGT"``, ``u32 ndim``, ``u32 dims[ndim]``, then little-endian f64.

Run it from the repository root once; its outputs are committed because the
reference tree does not exist where the GPU code runs::

    python ptarmigan_gb300/tables/extract.py <path of the reference's source tree>
"""

import math
import os
import re
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

_NAMED = {
    "NEG_INFINITY": -math.inf,
    "INFINITY": math.inf,
    "LN_10": math.log(10.0),
    "LN_2": math.log(2.0),
    "PI": math.pi,
}

_TOKEN = re.compile(
    r"(?P<num>[0-9]+(?:\.[0-9]*)?(?:[eE][+-]?[0-9]+)?)(?:_?f64)?"
    r"|(?P<name>[A-Za-z_][A-Za-z_0-9]*(?:::[A-Za-z_][A-Za-z_0-9]*)*)"
    r"|(?P<op>[-+*/(),\[\]{}:])"
)


def _initializer(src, name):
    """Return the text between ``=`` and the terminating ``;`` of ``name``."""
    m = re.search(r"(?:static|const)\s+" + re.escape(name) + r"\s*:", src)
    if m is None:
        raise KeyError(name)
    eq = src.index("=", m.end())
    depth = 0
    for i in range(eq + 1, len(src)):
        c = src[i]
        if c in "[({":
            depth += 1
        elif c in "])}":
            depth -= 1
        elif c == ";" and depth == 0:
            return src[eq + 1:i]
    raise ValueError("unterminated initializer for " + name)


def _values(text):
    """Flatten an initializer into floats, in source order.

    Handles the forms that occur in the table files: plain literals, unary
    minus, ``a/b`` and ``a*b`` between literals or named constants, and
    struct-field labels (``coeff:``), which are skipped.
    """
    toks = []
    for m in _TOKEN.finditer(text):
        if m.group("num") is not None:
            toks.append(("v", float(m.group("num"))))
        elif m.group("name") is not None:
            last = m.group("name").split("::")[-1]
            if last in _NAMED:
                toks.append(("v", _NAMED[last]))
            else:
                toks.append(("n", last))
        else:
            toks.append(("o", m.group("op")))
    out = []
    i = 0
    while i < len(toks):
        kind, val = toks[i]
        if kind == "n":
            i += 1
            continue
        if kind == "o" and val == "-" and i + 1 < len(toks) and toks[i + 1][0] == "v":
            # unary minus (binary minus never occurs between table entries)
            toks[i + 1] = ("v", -toks[i + 1][1])
            i += 1
            continue
        if kind == "v":
            acc = val
            while i + 2 < len(toks) and toks[i + 1] in (("o", "/"), ("o", "*")):
                op = toks[i + 1][1]
                rhs_kind, rhs = toks[i + 2]
                if rhs_kind != "v":
                    break
                acc = acc / rhs if op == "/" else acc * rhs
                i += 2
            out.append(acc)
        i += 1
    return out


def read_table(root, rel, name, shape):
    with open(os.path.join(root, rel)) as f:
        src = f.read()
    vals = _values(_initializer(src, name))
    n = 1
    for d in shape:
        n *= d
    if len(vals) != n:
        raise ValueError("%s:%s has %d values, expected %d" % (rel, name, len(vals), n))
    return vals


def read_scalar(root, rel, name):
    with open(os.path.join(root, rel)) as f:
        src = f.read()
    vals = _values(_initializer(src, name))
    if len(vals) != 1:
        raise ValueError("%s:%s is not a scalar" % (rel, name))
    return vals[0]


# (C name, reference file, reference symbol, shape)
SMALL_TABLES = [
    ("GAUSS_16_NODES", "src/quadrature/tables.rs", "GAUSS_16_NODES", (16,)),
    ("GAUSS_16_WEIGHTS", "src/quadrature/tables.rs", "GAUSS_16_WEIGHTS", (16,)),
    ("GAUSS_32_NODES", "src/quadrature/tables.rs", "GAUSS_32_NODES", (32,)),
    ("GAUSS_32_WEIGHTS", "src/quadrature/tables.rs", "GAUSS_32_WEIGHTS", (32,)),
    ("GL_NODES", "src/quadrature/tables.rs", "GL_NODES", (32,)),
    ("GL_WEIGHTS", "src/quadrature/tables.rs", "GL_WEIGHTS", (32,)),
    # Airy-function series (a then n) and Gauss-Laguerre rules with t^(-+1/6) weights
    ("AIRY_SMALL_X", "src/special_functions/airy.rs", "AIRY_SMALL_X", (2, 20)),
    ("AIRY_PRIME_SMALL_X", "src/special_functions/airy.rs", "AIRY_PRIME_SMALL_X", (2, 20)),
    ("GL_M16_NODES_40", "src/special_functions/airy.rs", "GL_m1_6_NODES_40", (40,)),
    ("GL_M16_WEIGHTS_40", "src/special_functions/airy.rs", "GL_m1_6_WEIGHTS_40", (40,)),
    ("GL_M16_NODES_16", "src/special_functions/airy.rs", "GL_m1_6_NODES_16", (16,)),
    ("GL_M16_WEIGHTS_16", "src/special_functions/airy.rs", "GL_m1_6_WEIGHTS_16", (16,)),
    ("GL_M16_NODES_4", "src/special_functions/airy.rs", "GL_m1_6_NODES_4", (4,)),
    ("GL_M16_WEIGHTS_4", "src/special_functions/airy.rs", "GL_m1_6_WEIGHTS_4", (4,)),
    ("GL_P16_NODES_32", "src/special_functions/airy.rs", "GL_p1_6_NODES_32", (32,)),
    ("GL_P16_WEIGHTS_32", "src/special_functions/airy.rs", "GL_p1_6_WEIGHTS_32", (32,)),
    ("GL_P16_NODES_16", "src/special_functions/airy.rs", "GL_p1_6_NODES_16", (16,)),
    ("GL_P16_WEIGHTS_16", "src/special_functions/airy.rs", "GL_p1_6_WEIGHTS_16", (16,)),
    ("GL_P16_NODES_8", "src/special_functions/airy.rs", "GL_p1_6_NODES_8", (8,)),
    ("GL_P16_WEIGHTS_8", "src/special_functions/airy.rs", "GL_p1_6_WEIGHTS_8", (8,)),
    ("GL_P16_NODES_4", "src/special_functions/airy.rs", "GL_p1_6_NODES_4", (4,)),
    ("GL_P16_WEIGHTS_4", "src/special_functions/airy.rs", "GL_p1_6_WEIGHTS_4", (4,)),
    # LCFA quantum synchrotron emission
    ("LCFA_LN_H_CHI_TABLE", "src/lcfa/photon_emission/tables.rs", "LN_H_CHI_TABLE", (41, 2)),
    ("LCFA_CLASSICAL_SPECTRUM_TABLE", "src/lcfa/photon_emission/tables.rs", "CLASSICAL_SPECTRUM_TABLE", (41, 2)),
    # each CDF record is {coeff, power, table[31][2]} = 64 doubles
    ("LCFA_QUANTUM_CDF", "src/lcfa/photon_emission/tables.rs", "QUANTUM_CDF", (41, 64)),
    ("LCFA_HIGH_CHI_CDF", "src/lcfa/photon_emission/tables.rs", "HIGH_CHI_CDF", (32, 2)),
    ("LCFA_HIGH_CHI_PEAK_CDF", "src/lcfa/photon_emission/tables.rs", "HIGH_CHI_PEAK_CDF", (32, 2)),
    ("LCFA_Y_INFINITE_DELTA_CDF", "src/lcfa/photon_emission/tables.rs", "Y_INFINITE_DELTA_CDF", (64,)),
    ("LCFA_Y_CDF", "src/lcfa/photon_emission/tables.rs", "Y_CDF", (31, 64)),
    ("LCFA_GAUNT_FACTOR_TABLE", "src/lcfa/photon_emission/mod.rs", "GAUNT_FACTOR_TABLE", (25, 2)),
    # LCFA Breit-Wheeler auxiliary function T(chi), parallel and perpendicular
    ("LCFA_LN_T_CHI_TABLE", "src/lcfa/pair_creation/tables.rs", "LN_T_CHI_TABLE", (81, 3)),
]

SCALARS = [
    ("LCFA_PH_DELTA_LN_CHI", "src/lcfa/photon_emission/tables.rs", "DELTA_LN_CHI"),
    ("LCFA_PH_LN_CHI_MIN", "src/lcfa/photon_emission/tables.rs", "LN_CHI_MIN"),
    ("LCFA_PH_LN_CHI_STEP", "src/lcfa/photon_emission/tables.rs", "LN_CHI_STEP"),
    ("LCFA_PH_LN_DELTA_MIN", "src/lcfa/photon_emission/tables.rs", "LN_DELTA_MIN"),
    ("LCFA_PH_LN_DELTA_STEP", "src/lcfa/photon_emission/tables.rs", "LN_DELTA_STEP"),
    ("LCFA_PAIR_DELTA_LN_CHI", "src/lcfa/pair_creation/tables.rs", "DELTA_LN_CHI"),
    # grids of the LMA tables (the data are in data/*.ptgt)
    ("NLC_CL_MIN", "src/nonlinear_compton/cp/classical/rate_table.rs", "MIN"),
    ("NLC_CL_STEP", "src/nonlinear_compton/cp/classical/rate_table.rs", "STEP"),
    ("BW_CP_LN_MIN_A", "src/pair_creation/cp/total.rs", "LN_MIN_A"),
    ("BW_CP_LN_MIN_ETA", "src/pair_creation/cp/total.rs", "LN_MIN_ETA"),
    ("BW_CP_LN_A_STEP", "src/pair_creation/cp/total.rs", "LN_A_STEP"),
    ("BW_CP_LN_ETA_STEP", "src/pair_creation/cp/total.rs", "LN_ETA_STEP"),
    ("BW_LP_LN_MIN_A", "src/pair_creation/lp/tables/total.rs", "LN_MIN_A"),
    ("BW_LP_LN_MIN_ETA", "src/pair_creation/lp/tables/total.rs", "LN_MIN_ETA"),
    ("BW_LP_LN_A_STEP", "src/pair_creation/lp/tables/total.rs", "LN_A_STEP"),
    ("BW_LP_LN_ETA_STEP", "src/pair_creation/lp/tables/total.rs", "LN_ETA_STEP"),
    ("BW_LPM_LN_MIN_A", "src/pair_creation/lp/tables/mid_range/total.rs", "LN_MIN_A"),
    ("BW_LPM_LN_MAX_ETA_PRIME", "src/pair_creation/lp/tables/mid_range/total.rs", "LN_MAX_ETA_PRIME"),
    ("BW_LPM_LN_MIN_ETA_PRIME", "src/pair_creation/lp/tables/mid_range/total.rs", "LN_MIN_ETA_PRIME"),
    ("BW_LPM_LN_A_STEP", "src/pair_creation/lp/tables/mid_range/total.rs", "LN_A_STEP"),
    ("BW_LPM_ETA_PRIME_DENSITY", "src/pair_creation/lp/tables/mid_range/total.rs", "ETA_PRIME_DENSITY"),
]

# two-element grid constants [a, eta], written as NAME_0 and NAME_1
PAIRS = [
    ("NLC_LP_MIN", "src/nonlinear_compton/lp/rate_table.rs", "MIN"),
    ("NLC_LP_STEP", "src/nonlinear_compton/lp/rate_table.rs", "STEP"),
    ("NLC_LP_CDF_MIN", "src/nonlinear_compton/lp/cdf_table.rs", "MIN"),
    ("NLC_LP_CDF_STEP", "src/nonlinear_compton/lp/cdf_table.rs", "STEP"),
    ("NLC_CP_MIN", "src/nonlinear_compton/cp/tables/total.rs", "MIN"),
    ("NLC_CP_STEP", "src/nonlinear_compton/cp/tables/total.rs", "STEP"),
    ("BW_LP_CDF_MIN", "src/pair_creation/lp/tables/cdf.rs", "MIN"),
    ("BW_LP_CDF_STEP", "src/pair_creation/lp/tables/cdf.rs", "STEP"),
]


def _c_double(v):
    if v == -math.inf:
        return "(-PTG_TABLE_INF)"
    if v == math.inf:
        return "PTG_TABLE_INF"
    return repr(float(v))


def write_small_header(root, path):
    lines = [
        "/* Generated by ptarmigan_gb300/tables/extract.py from the numeric",
        " * literals of the ptarmigan v1.5.0 sources (file and symbol named above",
        " * each array).  Do not edit by hand: re-run the script instead.",
        " *",
        " * The includer defines PTG_TABLE_DECL (storage class and qualifiers)",
        " * before including; the default suits plain C/C++ host code. */",
        "#pragma once",
        "#ifndef PTG_TABLE_DECL",
        "#define PTG_TABLE_DECL static const",
        "#endif",
        "#ifndef PTG_TABLE_INF",
        "#define PTG_TABLE_INF (__builtin_inf())",
        "#endif",
        "",
    ]
    for cname, rel, sym in SCALARS:
        v = read_scalar(root, rel, sym)
        lines.append("/* %s :: %s */" % (rel, sym))
        lines.append("#define PTG_%s %s" % (cname, _c_double(v)))
    for cname, rel, sym in PAIRS:
        v = read_table(root, rel, sym, (2,))
        lines.append("/* %s :: %s */" % (rel, sym))
        lines.append("#define PTG_%s_0 %s" % (cname, _c_double(v[0])))
        lines.append("#define PTG_%s_1 %s" % (cname, _c_double(v[1])))
    lines.append("")
    for cname, rel, sym, shape in SMALL_TABLES:
        vals = read_table(root, rel, sym, shape)
        dims = "".join("[%d]" % d for d in shape)
        lines.append("/* %s :: %s */" % (rel, sym))
        lines.append("PTG_TABLE_DECL double PTG_%s%s = {" % (cname, dims))
        per = 4
        body = []
        for i in range(0, len(vals), per):
            body.append("    " + ", ".join(_c_double(v) for v in vals[i:i + per]) + ",")
        lines.extend(body)
        lines.append("};")
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines))


def write_ptgt(path, shape, vals):
    with open(path, "wb") as f:
        f.write(b"PTGT")
        f.write(struct.pack("<I", len(shape)))
        for d in shape:
            f.write(struct.pack("<I", d))
        f.write(struct.pack("<%dd" % len(vals), *vals))


def read_ptgt(path):
    """Read back a table written by :func:`write_ptgt` as (shape, list)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] != b"PTGT":
        raise ValueError("bad magic in " + path)
    nd = struct.unpack_from("<I", data, 4)[0]
    shape = struct.unpack_from("<%dI" % nd, data, 8)
    off = 8 + 4 * nd
    n = 1
    for d in shape:
        n *= d
    return tuple(shape), list(struct.unpack_from("<%dd" % n, data, off))


# Large tables used by the LMA rates and samplers.
LARGE_TABLES = [
    ("nlc_lp_rate", "src/nonlinear_compton/lp/rate_table.rs", "TABLE", (68, 61)),
    ("nlc_lp_cdf", "src/nonlinear_compton/lp/cdf_table.rs", "TABLE", (4148, 16, 2)),
    ("nlc_cp_rate", "src/nonlinear_compton/cp/tables/total.rs", "TABLE", (70, 61)),
    ("nlc_lp_classical_rate", "src/nonlinear_compton/lp/classical/rate_table.rs", "TABLE", (61,)),
    ("nlc_lp_classical_cdf", "src/nonlinear_compton/lp/classical/cdf_table.rs", "TABLE", (61, 16, 2)),
    ("nlc_cp_classical_rate", "src/nonlinear_compton/cp/classical/rate_table.rs", "TABLE", (61,)),
    ("nlc_cp_classical_cdf", "src/nonlinear_compton/cp/classical/cdf_table.rs", "TABLE", (61, 32, 2)),
    ("bw_cp_total", "src/pair_creation/cp/total.rs", "TABLE", (121, 74, 2)),
    ("bw_lp_total", "src/pair_creation/lp/tables/total.rs", "TABLE", (61, 25, 2)),
    ("bw_lp_cdf", "src/pair_creation/lp/tables/cdf.rs", "TABLE", (1525, 16, 3)),
    ("bw_lp_mid_total", "src/pair_creation/lp/tables/mid_range/total.rs", "TABLE", (157, 36, 2)),
]


def main(argv):
    if len(argv) != 2:
        sys.exit("usage: extract.py <path of the reference's source tree (the directory holding src/)>")
    root = argv[1]
    write_small_header(root, os.path.join(HERE, "ptg_tables_small.h"))
    data = os.path.join(HERE, "data")
    os.makedirs(data, exist_ok=True)
    for name, rel, sym, shape in LARGE_TABLES:
        if not os.path.exists(os.path.join(root, rel)):
            print("skip (absent):", rel)
            continue
        vals = read_table(root, rel, sym, shape)
        write_ptgt(os.path.join(data, name + ".ptgt"), shape, vals)
    print("wrote tables to", HERE)


if __name__ == "__main__":
    main(sys.argv)
