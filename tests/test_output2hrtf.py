"""HRTF/HRIR post-processing (mesh2hrtf_gb300/output2hrtf.py) on the CPU:
the reference's referencing and HRIR rules (mesh2hrtf/Output2HRTF/
reference_hrtfs.py, compute_hrirs.py) on a project whose evaluation-grid
pressure is the free field of the reference source itself, so that the HRTF
is exactly 1 and the HRIR a delayed unit impulse."""
import json
import os

import numpy as np
import pytest

from mesh2hrtf_gb300 import output2hrtf as o2h

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
    paths = o2h.output2hrtf(str(tmp_path))
    h = np.load(paths[0])
    hrtf = h["Data_Real"] + 1j * h["Data_Imag"]
    assert hrtf.shape == (12, max(1, len(areas)), 4)
    np.testing.assert_allclose(hrtf, 1.0, rtol=0, atol=1e-12)
    assert str(h["GLOBAL_SOFAConventions"]) == ("SimpleFreeFieldHRTF" if len(areas) == 2 else "GeneralTF")
    # HRIR: fs = 2 * 4 kHz, 0 Hz bin of 1: a unit impulse delayed by 30 cm of travel
    ir = np.load(paths[1])
    fs = int(ir["Data_SamplingRate"])
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
    ha = np.load(o2h.output2hrtf(str(tmp_path / "a"))[0])
    hb = np.load(o2h.output2hrtf(str(tmp_path / "b"))[0])
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
