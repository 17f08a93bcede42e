"""Reads the compiled-in tables back out of ``ptg_tables_small.h``.

The header is the single copy of the small tables (the C++ and CUDA code
include it); this parser lets Python code see the same numbers.
"""

import functools
import os
import re

import numpy as np

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ptg_tables_small.h")


@functools.lru_cache(maxsize=None)
def _parse():
    with open(HEADER) as f:
        text = f.read()
    tables = {}
    for m in re.finditer(r"PTG_TABLE_DECL double PTG_(\w+)((?:\[\d+\])+) = \{(.*?)\};", text, re.S):
        name, dims, body = m.group(1), m.group(2), m.group(3)
        shape = tuple(int(d) for d in re.findall(r"\[(\d+)\]", dims))
        body = body.replace("(-PTG_TABLE_INF)", "-inf").replace("PTG_TABLE_INF", "inf")
        vals = [float(v) for v in body.replace("\n", " ").split(",") if v.strip()]
        tables[name] = np.array(vals, dtype=np.float64).reshape(shape)
    scalars = {m.group(1): float(m.group(2)) for m in re.finditer(r"#define PTG_(\w+) (\S+)\n", text)
               if re.match(r"^[-+0-9.eE]+$", m.group(2))}
    return tables, scalars


def table(name):
    return _parse()[0][name]


def scalar(name):
    return _parse()[1][name]
