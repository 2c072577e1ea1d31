"""Project report from NumCalc's NC*.out files.

Restates Mesh2HRTF's ``write_output_report`` (``Output2HRTF/
write_output_report.py:8-96``, parsing ``:99-246``, checks ``:271-354``),
which Output2HRTF runs before it reads the results: per source a table of
every frequency step (file it came from, input check, convergence, Krylov
iterations, relative error, timings) written as
``Output2HRTF/report_source_<k>.csv``, and a list of the steps that were
not calculated, had bad input or did not converge, written as
``Output2HRTF/report_issues.txt`` when there are any.

The drop-in NumCalc prints the NC.out lines this parser reads in the
reference's words (``Step <n>,``, ``Frequency = <f> Hz``, the CGS line,
the four timing lines, the iteration-limit warning), so its runs report
like the reference's.  What is alike the reference on purpose: the column
names, the CSV number formats and the issue text (users and scripts read
them), and the rules below.

* A file without a step marker is a "fundamental" failure of that file.
* A step found in several files takes its values from the last file read;
  NC.out is read first and the other NC*.out files after it (the
  reference reads those in directory order, this module by name).
* A value not found stays -1; a step never found keeps -1 in every column
  and names the last file read, as the reference's table index does.
* A step section without its own ``Step <n>,`` line adds to the step before
  it (the reference's loop variable carries over); before any step it is
  skipped.
* No issues: at least one source has a readable file, no entry is -1, and
  every step passed the input check and converged.
"""
from __future__ import annotations

import glob
import json
import os
import re

import numpy as np

COLUMNS = ("frequency step", "frequency in Hz", "NC input file", "Input check passed", "Converged",
           "Num. iterations", "relative error", "Comp. time total", "Comp. time assembling",
           "Comp. time solving", "Comp. time post-proc.")

STEP_MARK = ">> S T E P   N U M B E R   A N D   F R E Q U E N C Y <<"
BAD_INPUT = "Too many integral points in the theta"
NOT_CONVERGED = "Maximum number of iterations is reached!"

_STEP = re.compile(r"Step (\d+),")
_FREQ = re.compile(r"Frequency = (\d+(?:\.\d+)?) Hz")
_ITER = re.compile(r"number of iterations = (\d+),")
_ERR = re.compile(r"relative error = (.+)")
# (column, NC.out label): the labels are padded to one width in NC.out
_TIMES = ((8, "Assembling the equation system"), (9, "Solving the equation system"),
          (10, "Post processing"), (7, "Total"))
_TIME = {col: re.compile(re.escape(label.ljust(39)) + r": (\d+)") for col, label in _TIMES}


def nc_out_files(source_dir):
    """NC*.out files of a source folder in reading order: NC.out first."""
    names = sorted(os.path.basename(p) for p in glob.glob(os.path.join(source_dir, "NC*.out")))
    if "NC.out" in names:
        names.remove("NC.out")
        names.insert(0, "NC.out")
    return names


def parse_sections(text):
    """{step: {column: value}} of one NC*.out text, or None when the text
    holds no step section (a fundamental failure)."""
    parts = text.split(STEP_MARK)
    if len(parts) == 1:
        return None
    steps, step = {}, None
    for sec in parts[1:]:
        m = _STEP.search(sec)
        if m:
            step = int(m.group(1))
        if step is None:
            continue
        row = steps.setdefault(step, {})
        m = _FREQ.search(sec)
        if m:
            row[1] = float(m.group(1))
        row[3] = 0 if BAD_INPUT in sec else 1
        row[4] = 0 if NOT_CONVERGED in sec else 1
        m = _ITER.search(sec)
        if m:
            row[5] = int(m.group(1))
        m = _ERR.search(sec)
        if m:
            try:
                row[6] = float(m.group(1))
            except ValueError:
                pass
        for col, rx in _TIME.items():
            m = rx.search(sec)
            if m:
                row[col] = float(m.group(1))
    return steps


def source_table(source_dir, num_frequencies):
    """(file names, fundamental flag per file, table of shape
    (num_frequencies, 11)) of one source folder."""
    files = nc_out_files(source_dir)
    table = -np.ones((num_frequencies, len(COLUMNS)))
    table[:, 0] = np.arange(1, num_frequencies + 1)
    fundamentals = []
    for ff, name in enumerate(files):
        with open(os.path.join(source_dir, name)) as fh:
            steps = parse_sections(fh.read())
        fundamentals.append(steps is None)
        for step, row in (steps or {}).items():
            if not 1 <= step <= num_frequencies:
                continue
            table[step - 1, 2] = ff
            for col, v in row.items():
                table[step - 1, col] = v
    return files, fundamentals, table


def format_csv(files, table):
    """The report_source_<k>.csv text of one source."""
    lines = [", ".join(COLUMNS)]
    for r in table:
        name = files[int(r[2])] if files else ""
        lines.append("%d, %r, %s,%d, %d, %d, %r, %d, %d, %d, %d" % (
            int(r[0]), float(r[1]), name, int(r[3]), int(r[4]), int(r[5]), float(r[6]), int(r[7]), int(r[8]),
            int(r[9]), int(r[10])))
    return "\n".join(lines) + "\n"


def issues_text(tables):
    """The issue report for all sources' tables ("" when a source-level
    list is empty for every source, in which case the caller reports
    unknown issues)."""
    out = []
    for ss, t in enumerate(tables):
        missing = [int(r[0]) for r in t if r[1] == -1]
        seen = [r for r in t if r[1] != -1]
        bad = [int(r[0]) for r in seen if r[3] == 0]
        diverged = [int(r[0]) for r in seen if r[4] == 0]
        if not (missing or bad or diverged):
            continue
        out.append("Detected issues for source %d\n----------------------------\n" % (ss + 1))
        for title, steps in (("Frequency steps that were not calculated:", missing),
                             ("Frequency steps with bad input:", bad),
                             ("Frequency steps that did not converge:", diverged)):
            if steps:
                out.append("%s\n%s\n\n" % (title, ", ".join(str(s) for s in steps)))
    return "".join(out)


def write_output_report(folder=None):
    """Write the project report of a Mesh2HRTF project folder; returns
    (found_issues, report), report None when there are none."""
    folder = os.getcwd() if folder is None else folder
    with open(os.path.join(folder, "parameters.json")) as fh:
        num_frequencies = int(json.load(fh)["numFrequencies"])
    sources = glob.glob(os.path.join(folder, "NumCalc", "source_*"))
    sources.sort(key=lambda p: int(p.rsplit("_", 1)[-1]))
    out_dir = os.path.join(folder, "Output2HRTF")
    os.makedirs(out_dir, exist_ok=True)
    fundamentals, tables = [], []
    for ss, src in enumerate(sources):
        files, fund, table = source_table(src, num_frequencies)
        fundamentals.append(fund)
        tables.append(table)
        with open(os.path.join(out_dir, "report_source_%d.csv" % (ss + 1)), "w") as fh:
            fh.write(format_csv(files, table))
    all_broken = all(all(f) for f in fundamentals)
    clean = (not all_broken and not any((t == -1).any() for t in tables)
             and all(t[:, 3:5].all() for t in tables))
    if clean:
        return False, None
    report = issues_text(tables) or ("\nDetected unknown issues\n-----------------------\n"
                                     "Check the project reports in Output2HRTF,\n"
                                     "and the NC*.out files in NumCalc/source_*\n\n")
    report += ("For more information check Output2HRTF/report_source_*.csv "
               "and the NC*.out files located at NumCalc/source_*")
    with open(os.path.join(out_dir, "report_issues.txt"), "w") as fh:
        fh.write(report)
    return True, report
