"""SOFA (AES69) files for the HRTFs and HRIRs of a Mesh2HRTF project.

Mesh2HRTF writes its results with sofar (``Output2HRTF/output2hrtf.py:
209-287``, ``_get_sofa_object``, then ``sofar.write_sofa``).  sofar stores
SOFA in a netCDF-4 container (HDF5), and neither sofar nor an HDF5 or
netCDF-4 library is installed with this package.  This module writes the
same SOFA content (the conventions' dimensions, variables and attributes,
with the values Mesh2HRTF sets) in the netCDF classic container (64-bit
offset format) through ``scipy.io.netcdf_file``.  The netCDF library, and
thus sofar and the SOFA toolboxes built on it, open both containers through
the same calls; tools that parse HDF5 directly need the netCDF-4 one.

The SOFA object is a dict keyed as sofar names its attributes:
``GLOBAL_<name>`` for global attributes, the variable name for a variable
(``Data_Real`` for ``Data.Real``), and ``<variable>_<name>`` for a
variable's attribute (``SourcePosition_Units``).

Conventions (dimensions: M measurements, R receivers, E emitters, N
frequencies or samples, I = 1, C = 3):

=====================  ========  ============================================
convention             version   data
=====================  ========  ============================================
SimpleFreeFieldHRTF    1.0       Data.Real, Data.Imag (M, R, N); N (N)
GeneralTF              2.0       Data.Real, Data.Imag (M, R, N); N (N)
SimpleFreeFieldHRIR    1.0       Data.IR (M, R, N); Data.SamplingRate (I);
                                 Data.Delay (I, R)
GeneralFIR             1.0       as SimpleFreeFieldHRIR
=====================  ========  ============================================

Every convention also carries ListenerPosition (I, C), ListenerUp (I, C),
ListenerView (I, C), ReceiverPosition (R, C, I), SourcePosition (M, C) and
EmitterPosition (E, C, I); the FIR ones also SourceUp and SourceView (I, C).
The variables, their attributes and the global attributes of the two
SimpleFreeField conventions are the ones of the reference's SOFA files for
its SHTF test project (``tests/resources/SHTF/Output2HRTF``).
"""
from __future__ import annotations

import datetime

import numpy as np
from scipy.io import netcdf_file

API_VERSION = "1.1"        # the library's version (bem_version)


CONVENTIONS = {
    "SimpleFreeFieldHRTF": ("1.0", "TF"),
    "GeneralTF": ("2.0", "TF"),
    "SimpleFreeFieldHRIR": ("1.0", "FIR"),
    "GeneralFIR": ("1.0", "FIR"),
}

# variable -> dimensions (by the variable's sofar name)
_DIMS = {
    "ListenerPosition": ("I", "C"),
    "ListenerUp": ("I", "C"),
    "ListenerView": ("I", "C"),
    "ReceiverPosition": ("R", "C", "I"),
    "SourcePosition": ("M", "C"),
    "SourceUp": ("I", "C"),
    "SourceView": ("I", "C"),
    "EmitterPosition": ("E", "C", "I"),
    "Data_Real": ("M", "R", "N"),
    "Data_Imag": ("M", "R", "N"),
    "N": ("N",),
    "Data_IR": ("M", "R", "N"),
    "Data_SamplingRate": ("I",),
    "Data_Delay": ("I", "R"),
}

_GLOBAL_ORDER = ("Conventions", "Version", "SOFAConventions", "SOFAConventionsVersion", "APIName",
                 "APIVersion", "ApplicationName", "ApplicationVersion", "AuthorContact", "Comment",
                 "DataType", "DatabaseName", "DateCreated", "DateModified", "History", "License",
                 "ListenerShortName", "Organization", "Origin", "References", "RoomType", "Title")


def _nc_name(key):
    """File name of a variable: sofar's Data_X is Data.X."""
    return "Data." + key[5:] if key.startswith("Data_") else key


def new(convention):
    """An empty SOFA object of a convention with its default attributes and
    the default listener, emitter and orientation variables."""
    if convention not in CONVENTIONS:
        raise ValueError("convention must be one of %s" % ", ".join(CONVENTIONS))
    version, data_type = CONVENTIONS[convention]
    now = datetime.datetime.now().strftime("%Y-%m-%d %H:%M:%S")
    s = {
        "GLOBAL_Conventions": "SOFA", "GLOBAL_Version": "2.0", "GLOBAL_SOFAConventions": convention,
        "GLOBAL_SOFAConventionsVersion": version,
        "GLOBAL_APIName": "mesh2hrtf_gb300 SOFA writer (netCDF classic container)",
        "GLOBAL_APIVersion": API_VERSION, "GLOBAL_ApplicationName": "", "GLOBAL_ApplicationVersion": "",
        "GLOBAL_AuthorContact": "", "GLOBAL_Comment": "", "GLOBAL_DataType": data_type,
        "GLOBAL_DatabaseName": "", "GLOBAL_DateCreated": now, "GLOBAL_DateModified": now,
        "GLOBAL_History": "", "GLOBAL_License": "No license provided, ask the author for permission",
        "GLOBAL_ListenerShortName": "", "GLOBAL_Organization": "", "GLOBAL_Origin": "",
        "GLOBAL_References": "", "GLOBAL_RoomType": "free field", "GLOBAL_Title": "",
        "ListenerPosition": np.zeros((1, 3)), "ListenerPosition_Type": "cartesian",
        "ListenerPosition_Units": "metre",
        "ListenerUp": np.array([[0.0, 0.0, 1.0]]),
        "ListenerView": np.array([[1.0, 0.0, 0.0]]), "ListenerView_Type": "cartesian",
        "ListenerView_Units": "metre",
        "EmitterPosition": np.zeros((1, 3, 1)), "EmitterPosition_Type": "cartesian",
        "EmitterPosition_Units": "metre",
    }
    if data_type == "FIR":
        s.update({"SourceUp": np.array([[0.0, 0.0, 1.0]]), "SourceView": np.array([[1.0, 0.0, 0.0]]),
                  "SourceView_Type": "cartesian", "SourceView_Units": "metre",
                  "Data_SamplingRate_Units": "hertz"})
    else:
        s.update({"N_LongName": "frequency", "N_Units": "hertz"})
    return s


def _variables(sofa):
    return [k for k in sofa if not k.startswith("GLOBAL_") and k in _DIMS]


def _owner(key, variables):
    """(variable, attribute) of an attribute key, by the longest variable
    name that prefixes it."""
    best = None
    for v in variables:
        if key.startswith(v + "_") and (best is None or len(v) > len(best)):
            best = v
    if best is None:
        raise ValueError("%s is neither a SOFA variable nor an attribute of one" % key)
    return best, key[len(best) + 1:]


def dimensions(sofa):
    """{dimension: length} implied by the object's variables; raises if two
    variables disagree."""
    dims = {"I": 1, "C": 3}
    for k in _variables(sofa):
        shape = np.shape(sofa[k])
        names = _DIMS[k]
        if len(shape) != len(names):
            raise ValueError("%s has shape %s, expected dimensions %s" % (k, shape, names))
        for d, n in zip(names, shape):
            if dims.setdefault(d, n) != n:
                raise ValueError("dimension %s: %s has %d, another variable %d" % (d, k, n, dims[d]))
    return dims


def write(path, sofa):
    """Write a SOFA object (a dict from :func:`new`, filled) to ``path``."""
    variables = _variables(sofa)
    missing = [v for v in ("ReceiverPosition", "SourcePosition") if v not in sofa]
    conv = sofa.get("GLOBAL_SOFAConventions")
    data = ("Data_Real", "Data_Imag", "N") if CONVENTIONS.get(conv, (0, "TF"))[1] == "TF" \
        else ("Data_IR", "Data_SamplingRate", "Data_Delay")
    missing += [v for v in data if v not in sofa]
    if missing:
        raise ValueError("missing SOFA variables: %s" % ", ".join(missing))
    dims = dimensions(sofa)
    with netcdf_file(path, "w", version=2) as f:
        for k in _GLOBAL_ORDER:
            if "GLOBAL_" + k in sofa:
                setattr(f, k, _chars(sofa["GLOBAL_" + k]))
        for k, v in sofa.items():
            if k.startswith("GLOBAL_") and k[7:] not in _GLOBAL_ORDER:
                setattr(f, k[7:], _chars(v))
        for d in ("M", "R", "E", "N", "I", "C"):
            if d in dims:
                f.createDimension(d, dims[d])
        ncv = {}
        for k in variables:
            ncv[k] = f.createVariable(_nc_name(k), "d", _DIMS[k])
            ncv[k][:] = np.asarray(sofa[k], float)
        for k, v in sofa.items():
            if k.startswith("GLOBAL_") or k in _DIMS:
                continue
            var, attr = _owner(k, variables)
            setattr(ncv[var], attr, _chars(v))


def _chars(v):
    """A text attribute as netCDF characters: UTF-8 bytes, which the netCDF
    library reads back as the same string."""
    return str(v).encode("utf-8")


def _text(v):
    return v.decode("utf-8") if isinstance(v, bytes) else v


def read(path):
    """A SOFA object (dict) from a file :func:`write` made (or any SOFA file
    in the netCDF classic container)."""
    out = {}
    with netcdf_file(path, "r", mmap=False) as f:
        for k, v in f._attributes.items():
            out["GLOBAL_" + k] = _text(v)
        for name, var in f.variables.items():
            key = name.replace(".", "_")
            out[key] = np.array(var[:], float)
            for a, v in var._attributes.items():
                out[key + "_" + a] = _text(v)
    return out
