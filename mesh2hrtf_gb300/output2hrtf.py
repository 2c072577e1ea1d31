"""HRTFs and HRIRs from NumCalc results: the reference's Output2HRTF math.

Restates, for the traditional-BEM results this build produces:

* reading the evaluation-grid pressure of every source and frequency
  (``mesh2hrtf/Output2HRTF/output2hrtf.py:185-206,290-363``);
* referencing to the free-field pressure of the source placed at the origin
  (``reference_hrtfs.py:5-106``: point source, or the ear sources "Left ear",
  "Right ear", "Both ears" with volume flow 0.1 * area);
* HRIRs by the inverse real FFT of the conjugated, referenced spectrum with a
  0 Hz bin of 1, a real Nyquist bin and a circular shift of 30 cm of travel
  (``compute_hrirs.py:6-109``, ``output2hrtf.py:118-128``);
* the SOFA objects of ``_get_sofa_object`` (``output2hrtf.py:209-287``):
  evaluation points as spherical source positions (azimuth, elevation in
  degrees, radius), the ear positions (``sourceCenter``) as receivers,
  SimpleFreeFieldHRTF / HRIR for two receivers, GeneralTF / FIR otherwise.

The in-memory entry points (``hrtf_sofa``, ``write_hrtf_sofa``) take the
evaluation-grid pressure as the solver returns it (``capi.Solver.
solve_frequency``, ``capi.solve_batch``, ``capi.Server.wait``), so HRTFs come
straight from the results with no result file in between; ``output2hrtf``
reads a project's result files and calls them.

Differences from the reference:

* Results are read at full precision when the drop-in wrote them
  (``NUMCALC_GB300_NPY=1``: ``be.out/be.<k>/<name>.npy``); otherwise from the
  7-digit text files, as the reference does.
* The SOFA files are written by ``mesh2hrtf_gb300.sofa`` in the netCDF
  classic container (sofar, which writes netCDF-4/HDF5, is not installed);
  the conventions' variables and attributes are sofar's.
* Each grid's rows are selected by node id, not by the order of
  ``os.listdir(EvaluationGrids)``.

    python -m mesh2hrtf_gb300.output2hrtf <project folder>
"""
from __future__ import annotations

import json
import os
import sys
import warnings

import numpy as np

from . import output_report as _report
from . import project as _project
from . import sofa as _sofa


def read_result(step_dir, name, full_precision=True):
    """(ids, values) of be.out/be.<k>/<name>; values from <name>.npy when
    present and full_precision, else from the text file."""
    ids, vals = _project.read_result(os.path.join(step_dir, name))
    npy = os.path.join(step_dir, name + ".npy")
    if full_precision and os.path.isfile(npy):
        full = np.load(npy)
        if full.shape[0] != len(ids):
            raise ValueError("%s: %d rows in the .npy file, %d in the text file" % (step_dir, full.shape[0], len(ids)))
        vals = full
    return ids, vals


def read_pressure(folder, num_sources, num_frequencies, data="pEvalGrid", full_precision=True):
    """Pressure (or velocity) of all sources and steps: (ids, array of shape
    (points, sources, frequencies)), like _read_numcalc_data."""
    out, ids0 = [], None
    for s in range(num_sources):
        per = []
        for k in range(num_frequencies):
            d = os.path.join(folder, "NumCalc", "source_%d" % (s + 1), "be.out", "be.%d" % (k + 1))
            ids, vals = read_result(d, data, full_precision)
            if ids0 is None:
                ids0 = ids
            elif not np.array_equal(ids, ids0):
                raise ValueError("node ids differ between %s and the first result" % d)
            per.append(vals)
        out.append(np.stack(per, axis=-1))
    return ids0, np.stack(out, axis=1)


def cartesian_to_spherical(xyz):
    """Azimuth (0..360), elevation (-90..90) in degrees and radius, as
    _get_sofa_object converts the evaluation grid."""
    xyz = np.asarray(xyz, float)
    r = np.sqrt(np.sum(xyz ** 2, axis=1))
    z_div_r = np.where(r != 0, xyz[:, 2] / np.where(r != 0, r, 1.0), 0.0)
    el = 90 - np.arccos(z_div_r) / np.pi * 180
    az = np.mod(np.arctan2(xyz[:, 1], xyz[:, 0]), 2 * np.pi) / np.pi * 180
    return np.stack([az, el, r], axis=-1)


def reference_hrtfs(pressure, frequencies, radius, source_type, source_area, speed_of_sound, density,
                    mode="min"):
    """Pressure (points, receivers, frequencies) divided by the free-field
    pressure of the source at the origin (reference_hrtfs.py:66-103)."""
    p = np.asarray(pressure, complex)
    f = np.asarray(frequencies, float)
    radius = np.asarray(radius, float)
    if mode == "min":
        r = np.min(radius)
    elif mode == "mean":
        r = np.mean(radius)
    elif mode == "max":
        r = np.max(radius)
    else:
        r = radius[..., np.newaxis, np.newaxis]
    if source_type in ("Both ears", "Left ear", "Right ear"):
        flow = 0.1 * np.ones(p.shape)
        for nn in range(len(source_area)):
            flow[:, nn, :] = flow[:, nn, :] * source_area[nn]
        # point source in the origin evaluated at r (Williams, Fourier Acoustics, eq. 6.71)
        ps = -1j * density * 2 * np.pi * f * flow / (4 * np.pi) * np.exp(1j * 2 * np.pi * f / speed_of_sound * r) / r
    elif source_type == "Point source":
        ps = 0.1 * np.exp(1j * 2 * np.pi * f / speed_of_sound * r) / (4 * np.pi * r)
    elif source_type == "Plane wave":
        raise ValueError("Plane wave not implemented yet.")
    else:
        raise ValueError("Referencing is only implemented for sourceType 'Both ears', 'Left ear', 'Right ear', "
                         "'Point source' and 'Plane wave'.")
    return p / ps


def compute_hrirs(hrtf, frequencies, n_shift, sampling_rate=None):
    """(hrir, sampling_rate) from referenced HRTFs on f_1 .. f_max in equal
    steps (compute_hrirs.py:67-101)."""
    f = np.asarray(frequencies, float)
    if np.any(np.abs(np.diff(f, 2)) > .1) or f[0] < .1:
        raise ValueError("The frequency vector must go from f_1 > 0 to f_2 (half the sampling rate) in "
                         "equidistant steps.")
    p = np.array(hrtf, complex)
    if sampling_rate is None:
        sampling_rate = round(2 * f[-1])
    else:
        idx = int(np.argmin(np.abs(2 * f - sampling_rate)))
        if np.abs(2 * f[idx] - sampling_rate) > 1e-6:
            raise ValueError("The specified sampling rate is invalid. It must be two times any frequency for which "
                             "the HRTF was computed.")
        p = p[..., :idx + 1]
    p = np.concatenate((np.ones(p.shape[:-1] + (1,)), p), axis=-1)
    p[..., -1] = np.abs(p[..., -1])
    hrir = np.fft.irfft(np.conj(p))
    return np.roll(hrir, n_shift, axis=-1), sampling_rate


def _grid_nodes(folder, grid):
    nodes = np.loadtxt(os.path.join(folder, "EvaluationGrids", grid, "Nodes.txt"), skiprows=1, ndmin=2)
    return nodes[:, 0].astype(np.int64), nodes[:, 1:4]


def sofa_object(data, source_position, receiver_position, mode, mesh2hrtf_version, frequencies=None,
                sampling_rate=None):
    """The SOFA object of complex pressures or impulse responses of shape
    (points, receivers, frequencies or samples), as _get_sofa_object builds
    it (output2hrtf.py:209-287): the evaluation points (Cartesian) as
    spherical source positions, the ear positions as receivers."""
    data = np.asarray(data)
    n_rec = data.shape[1]
    if mode == "HRTF":
        conv = "SimpleFreeFieldHRTF" if n_rec == 2 else "GeneralTF"
    else:
        conv = "SimpleFreeFieldHRIR" if n_rec == 2 else "GeneralFIR"
    s = _sofa.new(conv)
    s["GLOBAL_ApplicationName"] = "Mesh2HRTF"
    s["GLOBAL_ApplicationVersion"] = str(mesh2hrtf_version)
    s["GLOBAL_History"] = "numerically simulated data"
    s["SourcePosition"] = cartesian_to_spherical(source_position)
    s["SourcePosition_Units"] = "degree, degree, meter"
    s["SourcePosition_Type"] = "spherical"
    s["ReceiverPosition"] = np.asarray(receiver_position, float).reshape(-1, 3, 1)
    s["ReceiverPosition_Units"] = "meter"
    s["ReceiverPosition_Type"] = "cartesian"
    if mode == "HRTF":
        s["Data_Real"] = np.real(data)
        s["Data_Imag"] = np.imag(data)
        s["N"] = np.asarray(frequencies, float).flatten()
    else:
        s["Data_IR"] = np.asarray(data, float)
        s["Data_SamplingRate"] = np.array([float(sampling_rate)])
        s["Data_Delay"] = np.zeros((1, n_rec))
    return s


def hrtf_sofa(pressure, grid_xyz, params):
    """(HRTF, HRIR) SOFA objects of one evaluation grid from its pressure
    (points, sources, frequencies) as the solver returned it, without a
    result file in between: the C ABI returns the potential, and the
    pressure is i * rho * omega times it (what the drop-in prints).  The
    HRIR object is None unless the project's ``computeHRIRs`` is set.
    ``params`` holds the keys of a project's parameters.json that
    Output2HRTF reads (output2hrtf.py:86-128)."""
    freqs = np.asarray(params["frequencies"], float)
    data = np.asarray(pressure, complex)
    if data.ndim != 3 or data.shape[0] != len(grid_xyz) or data.shape[2] != len(freqs):
        raise ValueError("pressure must have shape (points, sources, frequencies) = (%d, *, %d), not %s"
                         % (len(grid_xyz), len(freqs), data.shape))
    receivers = np.asarray(params["sourceCenter"], float).reshape(-1, 3)
    hrtf = sofa_object(data, grid_xyz, receivers, "HRTF", params.get("Mesh2HRTF_Version", ""), frequencies=freqs)
    if params.get("reference"):
        radius = hrtf["SourcePosition"][:, 2]
        data = reference_hrtfs(data, freqs, radius, params["sourceType"], params.get("sourceArea", []),
                               params["speedOfSound"], params["densityOfMedium"], mode="min")
        hrtf["Data_Real"], hrtf["Data_Imag"] = np.real(data), np.imag(data)
    hrir = None
    if params.get("computeHRIRs"):
        if not params.get("reference"):
            raise ValueError("Computing HRIRs requires prior referencing")
        fs = round(2 * freqs[-1])
        n_shift = int(np.round(.30 / (1 / fs * params["speedOfSound"])))
        ir, fs = compute_hrirs(data, freqs, n_shift)
        hrir = sofa_object(ir, grid_xyz, receivers, "HRIR", params.get("Mesh2HRTF_Version", ""),
                           sampling_rate=fs)
    return hrtf, hrir


def write_hrtf_sofa(out_dir, grid, pressure, grid_xyz, params):
    """Write ``HRTF_<grid>.sofa`` (and ``HRIR_<grid>.sofa`` with
    computeHRIRs) to out_dir from in-memory pressure; returns the paths."""
    os.makedirs(out_dir, exist_ok=True)
    hrtf, hrir = hrtf_sofa(pressure, grid_xyz, params)
    paths = [os.path.join(out_dir, "HRTF_%s.sofa" % grid)]
    _sofa.write(paths[0], hrtf)
    if hrir is not None:
        paths.append(os.path.join(out_dir, "HRIR_%s.sofa" % grid))
        _sofa.write(paths[1], hrir)
    return paths


def output2hrtf(folder, full_precision=True, report=True):
    """Process a project's NumCalc results (output2hrtf.py:15-128): the
    project report from the NC*.out files (a warning lists the issues; see
    output_report), then per evaluation grid the referenced HRTFs and, with
    computeHRIRs, the HRIRs, written as SOFA files to <folder>/Output2HRTF.
    Returns the SOFA paths written."""
    params_path = os.path.join(folder, "parameters.json")
    if not os.path.isfile(params_path):
        raise ValueError("The folder %s is not a valid Mesh2HRTF project. It must contain the file "
                         "'parameters.json'" % folder)
    with open(params_path) as fh:
        params = json.load(fh)
    out_dir = os.path.join(folder, "Output2HRTF")
    if report:
        found, text = _report.write_output_report(folder)
        if found:
            warnings.warn(text)
    ids, pressure = read_pressure(folder, params["numSources"], params["numFrequencies"], "pEvalGrid",
                                  full_precision)
    row_of = {int(i): r for r, i in enumerate(ids)}
    grids = params.get("evaluationGrids") or sorted(os.listdir(os.path.join(folder, "EvaluationGrids")))
    written = []
    for grid in grids:
        gid, xyz = _grid_nodes(folder, grid)
        rows = np.array([row_of[int(i)] for i in gid])
        written += write_hrtf_sofa(out_dir, grid, pressure[rows], xyz, params)
    return written


if __name__ == "__main__":
    for p in output2hrtf(sys.argv[1] if len(sys.argv) > 1 else os.getcwd()):
        print(p)
