"""Parameter flow of the reference: ``.ini`` -> ``input.txt`` -> parameters.

The reference flattens an ``.ini`` file into ``input.txt`` with
python/parser_ini.py:17-33 (one value per line, in the file's key order), and
its solver reads 17 values from ``input.txt`` in a fixed order
(src/read_input.cpp:24-72).  The key order in the ``.ini`` is therefore
load-bearing.  This module keeps that flow: ``ini_to_input_txt`` writes the
same ``input.txt`` the reference's script writes, and ``read_input`` reads it
the way the reference's ``read_input`` does (the host C++ driver has its own
reader, ``csrc/host/read_input.cpp``; the two are tested against each other).
"""
import configparser
import os

from ._abi import CbnsParams

# src/read_input.cpp:24-72, in order.
INPUT_ORDER = [
    ("checkpoint_fname", str), ("CFL", float), ("t_cur", float), ("t_end", float),
    ("Pr", float), ("gamma", float), ("Mach", float), ("Re", float), ("T_inf", float),
    ("L", float), ("IM", int), ("JM", int), ("KM", int), ("nstep_max", int),
    ("checkpoint_freq", int), ("num_output", int), ("is_restart", int),
]


def parse_ini(path):
    """(key, raw value) pairs of an ``.ini`` file in file order, keys case-kept
    (python/parser_ini.py:19-27)."""
    cfg = configparser.ConfigParser()
    cfg.optionxform = str
    if not cfg.read(path):
        raise FileNotFoundError(path)
    return [(k, cfg[sec][k]) for sec in cfg.sections() for k in cfg[sec]]


def ini_to_input_txt(ini_path, out_path="input.txt"):
    """Write ``input.txt`` from an ``.ini`` as python/parser_ini.py:29-33 does."""
    pairs = parse_ini(ini_path)
    with open(out_path, "w") as f:
        for _, v in pairs:
            f.write(v)
            f.write("\n")
    return pairs


def _token(v):
    if isinstance(v, bytes):
        return v.decode()
    if isinstance(v, float):
        return repr(v)
    return str(v)


def write_input_txt(params, out_path="input.txt"):
    """Write ``input.txt`` holding ``params`` (a CbnsParams) in read_input's order.
    Floats are written shortest-round-trip, so they read back bit-identical."""
    with open(out_path, "w") as f:
        for name, _ in INPUT_ORDER:
            f.write(_token(getattr(params, name)))
            f.write("\n")


def read_input(path="input.txt"):
    """Read ``input.txt`` as src/read_input.cpp:15-103 does and derive the
    constants of src/read_input.cpp:78-90.  Unlike the reference (whose
    try/catch never fires because the stream's exceptions are not enabled), a
    missing file or a short/unparsable one raises."""
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    with open(path) as f:
        toks = f.read().split()
    if len(toks) < len(INPUT_ORDER):
        raise ValueError("%s holds %d values, %d expected" % (path, len(toks), len(INPUT_ORDER)))
    p = CbnsParams()
    for (name, typ), tok in zip(INPUT_ORDER, toks):
        if typ is str:
            p.checkpoint_fname = tok.encode()[:255]
        elif typ is float:
            setattr(p, name, float(tok))
        else:
            setattr(p, name, int(tok))
    return p.derive()
