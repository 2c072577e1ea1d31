"""HRTF/HRIR post-processing (mesh2hrtf_gb300/output2hrtf.py, sofa.py) on
the CPU: the reference's referencing and HRIR rules (mesh2hrtf/Output2HRTF/
reference_hrtfs.py, compute_hrirs.py) on a project whose evaluation-grid
pressure is the free field of the reference source itself, so that the HRTF
is exactly 1 and the HRIR a delayed unit impulse; and the reference's own
SHTF test project against the SOFA files the reference wrote for it
(tests/golden/shtf_output2hrtf.npz, made by make_output2hrtf_golden.py)."""
import json
import os
import pathlib

import numpy as np
import pytest

from mesh2hrtf_gb300 import output2hrtf as o2h
from mesh2hrtf_gb300 import sofa

C, RHO = 343.0, 1.1839


def _write_result(path, ids, vals, npy):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        fh.write("Mesh2HRTF 1.0.0\n    1\n%5d %5d\n" % (7, len(ids)))
        for i, v in zip(ids, vals):
            fh.write("%5d % E % E\n" % (i, v.real, v.imag))
    if npy:
        np.save(path + ".npy", np.asarray(vals, np.complex128))


def _project(root, source_type, freqs, areas=(), npy=True, radius=1.0, reference=True, hrirs=True):
    rng = np.random.default_rng(5)
    d = rng.normal(size=(12, 3))
    xyz = d / np.linalg.norm(d, axis=1)[:, None] * radius
    ids = np.arange(300, 312)
    g = root / "EvaluationGrids" / "G"
    g.mkdir(parents=True)
    with open(g / "Nodes.txt", "w") as fh:
        fh.write("%d\n" % len(ids))
        for i, p in zip(ids, xyz):
            fh.write("%d %.17e %.17e %.17e\n" % (i, p[0], p[1], p[2]))
    nsrc = max(1, len(areas))
    params = {"Mesh2HRTF_Version": "1.0.0", "speedOfSound": C, "densityOfMedium": RHO,
              "evaluationGrids": ["G"], "sourceType": source_type, "numSources": nsrc,
              "sourceCenter": [[0.0, 0.09 * (1 - 2 * s), 0.0] for s in range(nsrc)],
              "sourceArea": list(areas), "reference": reference, "computeHRIRs": hrirs,
              "numFrequencies": len(freqs), "frequencies": list(freqs)}
    (root / "parameters.json").write_text(json.dumps(params))
    r = np.linalg.norm(xyz, axis=1)
    for s in range(nsrc):
        for k, f in enumerate(freqs):
            kk = 2 * np.pi * f / C
            if source_type == "Point source":
                p = 0.1 * np.exp(1j * kk * r) / (4 * np.pi * r)
            else:
                q = 0.1 * areas[s]
                p = -1j * RHO * 2 * np.pi * f * q / (4 * np.pi) * np.exp(1j * kk * r) / r
            _write_result(str(root / "NumCalc" / ("source_%d" % (s + 1)) / "be.out" / ("be.%d" % (k + 1)) /
                              "pEvalGrid"), ids, p, npy)
    return xyz


@pytest.mark.parametrize("source_type,areas", [("Point source", ()), ("Both ears", (3.2e-5, 3.7e-5)),
                                               ("Left ear", (3.2e-5,))])
def test_free_field_of_the_reference_source_gives_unit_hrtf(tmp_path, source_type, areas):
    freqs = [1000.0, 2000.0, 3000.0, 4000.0]
    _project(tmp_path, source_type, freqs, areas)
    paths = o2h.output2hrtf(str(tmp_path), report=False)
    assert [os.path.basename(p) for p in paths] == ["HRTF_G.sofa", "HRIR_G.sofa"]
    h = sofa.read(paths[0])
    hrtf = h["Data_Real"] + 1j * h["Data_Imag"]
    assert hrtf.shape == (12, max(1, len(areas)), 4)
    np.testing.assert_allclose(hrtf, 1.0, rtol=0, atol=1e-12)
    assert str(h["GLOBAL_SOFAConventions"]) == ("SimpleFreeFieldHRTF" if len(areas) == 2 else "GeneralTF")
    # HRIR: fs = 2 * 4 kHz, 0 Hz bin of 1: a unit impulse delayed by 30 cm of travel
    ir = sofa.read(paths[1])
    assert ir["GLOBAL_SOFAConventions"] == ("SimpleFreeFieldHRIR" if len(areas) == 2 else "GeneralFIR")
    fs = int(ir["Data_SamplingRate"][0])
    n_shift = int(np.round(.30 / (1 / fs * C)))
    assert fs == 8000 and n_shift == 7
    expect = np.zeros(8)
    expect[n_shift % 8] = 1.0
    np.testing.assert_allclose(ir["Data_IR"], np.broadcast_to(expect, ir["Data_IR"].shape), atol=1e-12)


def test_text_results_lose_digits_npy_results_do_not(tmp_path):
    freqs = [500.0, 1000.0]
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    _project(tmp_path / "a", "Point source", freqs, npy=True, hrirs=False)
    _project(tmp_path / "b", "Point source", freqs, npy=False, hrirs=False)
    ha = sofa.read(o2h.output2hrtf(str(tmp_path / "a"), report=False)[0])
    hb = sofa.read(o2h.output2hrtf(str(tmp_path / "b"), report=False)[0])
    ea = np.abs(ha["Data_Real"] + 1j * ha["Data_Imag"] - 1).max()
    eb = np.abs(hb["Data_Real"] + 1j * hb["Data_Imag"] - 1).max()
    assert ea < 1e-13 and 1e-9 < eb < 1e-5   # % E prints 7 significant digits


def test_source_positions_follow_the_sofa_convention(tmp_path):
    xyz = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 2.0], [-1.0, -1.0, 0]])
    sph = o2h.cartesian_to_spherical(xyz)
    np.testing.assert_allclose(sph, [[0, 0, 1], [90, 0, 1], [0, 90, 2], [225, 0, np.sqrt(2)]], atol=1e-12)


def test_hrir_rejects_uneven_frequencies():
    with pytest.raises(ValueError):
        o2h.compute_hrirs(np.ones((1, 1, 3)), [100.0, 200.0, 400.0], 0)
    with pytest.raises(ValueError):
        o2h.compute_hrirs(np.ones((1, 1, 3)), [100.0, 200.0, 300.0], 0, sampling_rate=500)
    hrir, fs = o2h.compute_hrirs(np.ones((1, 1, 3)), [100.0, 200.0, 300.0], 0, sampling_rate=400)
    assert fs == 400 and hrir.shape == (1, 1, 4)


# ------------------------------------------------ the reference's SHTF project
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "shtf_output2hrtf.npz")


def _shtf_project(root, g, params):
    grid = str(g["grid_name"])
    (root / "EvaluationGrids" / grid).mkdir(parents=True)
    with open(root / "EvaluationGrids" / grid / "Nodes.txt", "w") as fh:
        fh.write("%d\n" % len(g["grid_nodes"]))
        for r in g["grid_nodes"]:
            fh.write("%d %.6f %.6f %.6f\n" % (int(r[0]), r[1], r[2], r[3]))
    (root / "parameters.json").write_text(json.dumps(params))
    texts, nf = g["pEvalGrid_text"], params["numFrequencies"]
    for s in range(params["numSources"]):
        for k in range(nf):
            d = root / "NumCalc" / ("source_%d" % (s + 1)) / "be.out" / ("be.%d" % (k + 1))
            d.mkdir(parents=True)
            (d / "pEvalGrid").write_text(str(texts[s * nf + k]))
    return grid


def _as_run(g):
    """The project's parameters as the reference's run saw them: its SOFA
    files carry the ear positions at 6 decimals, and its HRTFs divided by
    ours with the parameters.json areas are a constant per ear, 1 - 8.6e-7
    and 1 - 1.2e-6, the relative change of rounding the areas to 6
    significant digits (the next test pins that ratio)."""
    params = json.loads(str(g["params_json"]))
    params["sourceCenter"] = g["HRTF__ReceiverPosition"][:, :, 0].tolist()
    params["sourceArea"] = [float("%.6g" % a) for a in params["sourceArea"]]
    return params


@pytest.mark.parametrize("kind", ["HRTF", "HRIR"])
def test_shtf_matches_the_reference_sofa_files(tmp_path, kind):
    """2 ear sources, 60 frequencies, 4 evaluation points read from the
    reference's be.out text files: every variable of the reference's SOFA
    file to 1e-14 and every attribute equal (but the writer's name and
    version and the dates)."""
    g = np.load(GOLDEN)
    grid = _shtf_project(tmp_path, g, _as_run(g))
    paths = o2h.output2hrtf(str(tmp_path), report=False)
    ours = sofa.read(paths[0 if kind == "HRTF" else 1])
    ref = {k[len(kind) + 2:]: g[k] for k in g.files if k.startswith(kind + "__") and "___dim_" not in k}
    assert set(ours) == set(ref)
    skip = {"GLOBAL_APIName", "GLOBAL_APIVersion", "GLOBAL_DateCreated", "GLOBAL_DateModified"}
    for k, v in ref.items():
        if k in skip:
            continue
        if v.dtype.kind == "U":
            assert ours[k] == str(v), k
        else:
            assert ours[k].shape == v.shape, k
            np.testing.assert_allclose(ours[k], v, rtol=1e-14, atol=1e-14 * np.abs(v).max(), err_msg=k)
    dims = {k[len(kind) + 7:]: int(g[k]) for k in g.files if k.startswith(kind + "___dim_")}
    ours_dims = sofa.dimensions(ours)
    assert all(ours_dims[d] == n for d, n in dims.items() if d != "S")   # S: strings, none here
    assert os.path.basename(paths[0]) == "HRTF_%s.sofa" % grid


def test_shtf_with_the_committed_parameters_differs_by_the_area_rounding(tmp_path):
    g = np.load(GOLDEN)
    params = json.loads(str(g["params_json"]))
    _shtf_project(tmp_path, g, params)
    h = sofa.read(o2h.output2hrtf(str(tmp_path), report=False)[0])
    ratio = (h["Data_Real"] + 1j * h["Data_Imag"]) / (g["HRTF__Data_Real"] + 1j * g["HRTF__Data_Imag"])
    expect = np.array([float("%.6g" % a) / a for a in params["sourceArea"]])
    np.testing.assert_allclose(ratio, np.broadcast_to(expect[None, :, None], ratio.shape), rtol=1e-13)


def test_in_memory_pressure_equals_the_file_path(tmp_path):
    """hrtf_sofa on the pressure array (as the solver returns it) gives the
    SOFA objects output2hrtf makes from the result files."""
    freqs = [1000.0, 2000.0, 3000.0, 4000.0]
    xyz = _project(tmp_path, "Both ears", freqs, (3.2e-5, 3.7e-5))
    params = json.loads((tmp_path / "parameters.json").read_text())
    ids, pressure = o2h.read_pressure(str(tmp_path), 2, len(freqs))
    files = [sofa.read(p) for p in o2h.output2hrtf(str(tmp_path), report=False)]
    mem = o2h.hrtf_sofa(pressure, xyz, params)
    for a, b in zip(mem, files):
        for k, v in a.items():
            if k.startswith("GLOBAL_Date"):
                continue
            if isinstance(v, str):
                assert b[k] == v, k
            else:
                np.testing.assert_array_equal(np.asarray(v, float), b[k], err_msg=k)
    with pytest.raises(ValueError):
        o2h.hrtf_sofa(pressure[:, :, :3], xyz, params)


def test_sofa_round_trip_and_checks(tmp_path):
    s = sofa.new("GeneralTF")
    assert s["GLOBAL_DataType"] == "TF" and s["GLOBAL_SOFAConventionsVersion"] == "2.0"
    rng = np.random.default_rng(1)
    s.update(Data_Real=rng.normal(size=(5, 1, 3)), Data_Imag=rng.normal(size=(5, 1, 3)), N=[1.0, 2.0, 3.0],
             SourcePosition=rng.normal(size=(5, 3)), ReceiverPosition=np.zeros((1, 3, 1)),
             SourcePosition_Type="spherical", GLOBAL_Comment="x", GLOBAL_AuthorContact="Jörg Müller")
    path = str(tmp_path / "a.sofa")
    sofa.write(path, s)
    assert pathlib.Path(path).read_bytes()[:4] == b"CDF\x02"          # netCDF classic, 64-bit offsets
    r = sofa.read(path)
    assert set(r) == set(s)
    for k, v in s.items():
        if isinstance(v, str):
            assert r[k] == v
        else:
            np.testing.assert_array_equal(r[k], np.asarray(v, float))
    assert sofa.dimensions(r) == {"I": 1, "C": 3, "M": 5, "R": 1, "N": 3, "E": 1}
    bad = dict(s, Data_Imag=np.zeros((5, 1, 4)))
    with pytest.raises(ValueError):
        sofa.write(str(tmp_path / "b.sofa"), bad)
    with pytest.raises(ValueError):
        sofa.write(str(tmp_path / "c.sofa"), {k: v for k, v in s.items() if k != "N"})
    with pytest.raises(ValueError):
        sofa.write(str(tmp_path / "d.sofa"), dict(s, Bogus_Units="m"))
    with pytest.raises(ValueError):
        sofa.new("FreeFieldDirectivityTF")


def test_shtf_output2hrtf_writes_the_reference_reports(tmp_path):
    """The whole of Output2HRTF on the SHTF project with its NC*.out files:
    the reports equal the reference's (no issues, so no warning) and the
    SOFA files are written."""
    import warnings

    g = np.load(GOLDEN)
    _shtf_project(tmp_path, g, _as_run(g))
    rep = json.loads(str(np.load(os.path.join(os.path.dirname(__file__), "golden", "output_report.npz"))["doc"]))
    for s, files in enumerate(rep["SHTF"]["files"]):
        for name, text in files.items():
            (tmp_path / "NumCalc" / ("source_%d" % (s + 1)) / name).write_text(text)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        paths = o2h.output2hrtf(str(tmp_path))
    assert len(paths) == 2
    for s, ref in enumerate(rep["SHTF"]["csv"]):
        assert (tmp_path / "Output2HRTF" / ("report_source_%d.csv" % (s + 1))).read_text() == ref
    assert not (tmp_path / "Output2HRTF" / "report_issues.txt").exists()


def test_missing_steps_warn(tmp_path):
    _project(tmp_path, "Point source", [500.0, 1000.0], hrirs=False)
    with pytest.warns(UserWarning, match="Frequency steps that were not calculated:\n1, 2"):
        o2h.output2hrtf(str(tmp_path))
