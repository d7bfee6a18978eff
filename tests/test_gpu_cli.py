"""psdbscan end to end: TSV in -> clustering on the GPU -> TSV out, checked
against the oracle on the rows that survive the empty-value deletion
(cpp/TableHolder.hpp:283-285) -- including the empty row the reader appends for
the file's final newline (cpp/csvreader.hpp:152-180)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import build, synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _write_inputs(tmp_path, w, hamming, noise):
    vg = tmp_path / "VHgenes.txt"
    jg = tmp_path / "JHgenes.txt"
    vg.write_bytes(b"\n".join(w.v_genes) + b"\n\n")
    jg.write_bytes(b"\n".join(w.j_genes) + b"\n")
    conf = open(os.path.join(ROOT, "tests", "golden", "psdbscan_test.conf")).read()
    conf = (conf.replace("@VGENES@", str(vg)).replace("@JGENES@", str(jg))
            .replace("@HAMMING@", "true" if hamming else "false")
            .replace("@NOISE@", "true" if noise else "false"))
    cf = tmp_path / "test.conf"
    cf.write_text(conf)
    rows = [b"Sequence number\tSequence ID\tV-GENE and allele\tJ-GENE and allele\tCDR3-IMGT\tExtra"]
    keep = []
    for i in range(w.n):
        v, j, s = w.vcall(i), w.jcall(i), w.seq(i)
        if i % 97 == 5:
            s = b""          # deleted: empty sequence
        if i % 89 == 7:
            v = b""          # deleted: empty V call
        rows.append(b"%d\tid%d\t%s\t%s\t%s\tx" % (i, i, v, j, s))
        if s and v and j:
            keep.append(i)
    inp = tmp_path / "repertoire.tsv"
    inp.write_bytes(b"\n".join(rows) + b"\n")
    return cf, inp, keep


@pytest.mark.parametrize("hamming,noise", [(False, False), (True, True)])
def test_psdbscan_end_to_end(tmp_path, hamming, noise):
    w = synth.workload(0, scale=0.3)
    cf, inp, keep = _write_inputs(tmp_path, w, hamming, noise)
    r = subprocess.run([build.CLI, "--config_file", str(cf), "--input", str(inp)],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "output_repertoire.csv"
    lines = out.read_text().split("\n")
    assert lines[-1] == ""
    header = lines[0].split("\t")
    assert header == ["Original.Filename", "ID.code", "V_CALL", "CDR3", "Not.In.Input", "Cores",
                      "Copies", "Clone"]
    body = [l.split("\t") for l in lines[1:-1]]
    # oracle on the surviving rows, threshold 0.15 relative as configured
    sub = synth.take_rows(w, np.array(keep))
    sub.threshold, sub.abs_eps, sub.min_pts, sub.use_hamming = 0.15, -1, 2, hamming
    o = oracle.cluster(sub)
    want = [(str(int(o.core[k])), str(int(o.copies[k])), str(int(o.clone_id[k])))
            for k in range(len(keep))]
    ids = ["id%d" % i for i in keep]
    if noise:
        sel = [k for k in range(len(keep)) if o.clone_id[k] != 0]
        want = [want[k] for k in sel]
        ids = [ids[k] for k in sel]
    assert [b[1] for b in body] == ids
    assert [(b[5], b[6], b[7]) for b in body] == want
    assert all(b[4] == "" for b in body)
    assert all(b[0] == str(inp) for b in body)
    bench = (tmp_path / "benchmark_repertoire.csv").read_text().splitlines()
    assert bench[0] == "Timer/Message\tValue"
    assert any("Number of uniques = %d" % o.n_uniques in l for l in bench)
    assert any("Number of trees with depth 0" in l for l in bench)
