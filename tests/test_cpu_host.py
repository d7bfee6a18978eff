"""CPU-side checks: the kernels' integer helpers compiled as host code, the
C ABI library (loads, exports every declared symbol, reports a missing device),
and the Python mirror's argument handling."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "immunodbscan_gb300.h")


def test_bitops_host(tmp_path):
    exe = tmp_path / "test_bitops"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "immunodbscan_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "test_bitops.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:idb_status|size_t|const char \*|int)\s+\*?(idb_\w+)\(",
                                 text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["idb_cluster", "idb_cluster_device", "idb_batch_plan", "idb_batch_run",
              "idb_context_create", "idb_context_destroy", "idb_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    from immunodbscan_gb300 import _lib
    assert os.path.exists(_lib.LIB_PATH), "build the library first (__graft_entry__.build())"
    L = C.CDLL(_lib.LIB_PATH)
    for n in declared_functions():
        assert hasattr(L, n), f"{n} declared in the header but not exported"
    assert _lib.lib().idb_abi_version() == 1


def test_status_strings():
    from immunodbscan_gb300 import _lib
    for s in range(9):
        assert _lib.lib().idb_status_string(s)


def test_no_device_is_reported():
    """Without a GPU the library reports IDB_ERR_NO_DEVICE instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from immunodbscan_gb300 import IdbError, Context
    with pytest.raises(IdbError) as e:
        Context(0)
    assert e.value.status == 3


def test_interlink_rejects_bad_columns():
    from immunodbscan_gb300 import Interlink
    with pytest.raises(ValueError):
        Interlink([b"IGHV1*"], None, [b"CAR", b"CAK"], 2, [b"IGHV1*"], [], 0.1, 2, False)


def test_synthetic_workloads_shapes():
    from immunodbscan_gb300 import synth
    for k, scale in [(0, 0.1), (1, 0.01), (2, 0.002), (3, 0.002), (4, 0.0005)]:
        w = synth.workload(k, scale=scale)
        assert w.n == int(w.rep_off[-1])
        assert len(w.seq_off) == w.n + 1 and len(w.v_off) == w.n + 1
        L = w.lengths()
        assert L.min() >= 1
        if k == 1:
            assert np.all(L % 3 == 0)
    w = synth.workload(2, scale=0.002)
    assert w.n_rep == 64


def test_host_surface_cpp(tmp_path):
    """INFO reader, escaped_list_separator tokenizer, CSV reader/writer quirks."""
    exe = tmp_path / "test_host"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "immunodbscan_gb300", "host"),
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_host.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_parallel_csv_matches_serial(tmp_path):
    """The multi-threaded CSV reader and writer give the one-thread forms'
    tables and bytes (up to 200,000-row files, all of the reader's quirks)."""
    exe = tmp_path / "test_csv_parallel"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I",
                    os.path.join(ROOT, "immunodbscan_gb300", "host"),
                    os.path.join(ROOT, "tests", "cpp", "test_csv_parallel.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def _cli():
    from immunodbscan_gb300 import build
    return build.CLI


def test_psdbscan_help_and_errors(tmp_path):
    cli = _cli()
    assert os.path.exists(cli), "build the host first (__graft_entry__.build())"
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 1 and "--config_file" in r.stdout and "--input" in r.stdout
    r = subprocess.run([cli, "--config_file", str(tmp_path / "nope.conf")], capture_output=True,
                       text=True)
    assert r.returncode == 2 and "cannot open" in r.stderr
    r = subprocess.run([cli, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1


@pytest.mark.parametrize("noise", [False, True])
def test_psdbscan_table_flow_with_stand_in_library(tmp_path, noise):
    """The psdbscan host built against tests/cpp/fake_idb.cpp (row r of the
    clustered table gets clone r%3, core r%2, copies 1+r%4): rows with an empty
    sequence, V or J value are deleted before clustering, the read columns keep
    their values in row order, the results line up with the surviving rows,
    noise rows (clone 0) go when configured, an unread column is written empty."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_gpu_cli import _write_inputs
    from immunodbscan_gb300 import synth
    d = tmp_path / "bin"
    d.mkdir()
    inc = ["-I", os.path.join(ROOT, "include")]
    subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", *inc,
                    os.path.join(ROOT, "tests", "cpp", "fake_idb.cpp"), "-o",
                    str(d / "libimmunodbscan_gb300.so")], check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", *inc, "-I", os.path.join(ROOT, "immunodbscan_gb300", "host"),
                    os.path.join(ROOT, "immunodbscan_gb300", "host", "psdbscan.cpp"), "-o",
                    str(d / "psdbscan"), "-L" + str(d), "-limmunodbscan_gb300", "-Wl,-rpath,$ORIGIN"],
                   check=True)
    w = synth.workload(0, scale=0.05)
    cf, inp, keep = _write_inputs(tmp_path, w, False, noise)
    r = subprocess.run([str(d / "psdbscan"), "--config_file", str(cf), "--input", str(inp)],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    lines = (tmp_path / "output_repertoire.csv").read_text().split("\n")
    assert lines[0].split("\t") == ["Original.Filename", "ID.code", "V_CALL", "CDR3", "Not.In.Input",
                                    "Cores", "Copies", "Clone"]
    assert lines[-1] == ""
    body = [l.split("\t") for l in lines[1:-1]]
    want = [(k, i) for k, i in enumerate(keep) if not (noise and k % 3 == 0)]
    assert len(body) == len(want)
    for b, (k, i) in zip(body, want):
        assert b == [str(inp), "id%d" % i, w.vcall(i).decode(), w.seq(i).decode(), "",
                     str(k % 2), str(1 + k % 4), str(k % 3)]
    assert (tmp_path / "benchmark_repertoire.csv").exists()


def test_mlp_cpu_gradient_is_exact():
    """The NumPy reference gradient (used to check the device training kernel)
    against central finite differences."""
    from immunodbscan_gb300 import learned
    rng = np.random.default_rng(0)
    X = rng.normal(0, 1, size=(40, learned.F))
    T = rng.normal(5, 2, size=40)
    p = learned.init_params(1).astype(np.float64)
    g, _ = learned.cpu_grad(p, X, T)
    idx = rng.choice(len(p), size=60, replace=False)
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (np.mean((learned.forward(pp, X) - T) ** 2) -
              np.mean((learned.forward(pm, X) - T) ** 2)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd))


def test_params_and_stats_mirror_the_header():
    """The ctypes mirrors of idb_params and idb_stats follow the header's
    layout (the candidate-path fields included)."""
    import ctypes as C
    from immunodbscan_gb300 import _lib
    hdr = open(os.path.join(ROOT, "include", "immunodbscan_gb300.h")).read()
    assert "int32_t  candidates;" in hdr and "uint32_t candidates;" in hdr
    assert _lib.Params.candidates.offset == 8 * 4
    assert C.sizeof(_lib.Params) == 12 * 4
    assert _lib.Stats.candidates.offset == _lib.Stats.lev_columns.offset + 8
    assert C.sizeof(_lib.Stats) % 8 == 0


def test_psdbscan_candidate_pairs_key(tmp_path):
    """The optional INFO key candidate_pairs reaches idb_params.candidates
    ("buckets" -> 1; the stand-in library then reports copies 7 on every row),
    and an unknown value stops the host with a message."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_gpu_cli import _write_inputs
    from immunodbscan_gb300 import synth
    d = tmp_path / "bin"
    d.mkdir()
    inc = ["-I", os.path.join(ROOT, "include")]
    subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", *inc,
                    os.path.join(ROOT, "tests", "cpp", "fake_idb.cpp"), "-o",
                    str(d / "libimmunodbscan_gb300.so")], check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", *inc, "-I", os.path.join(ROOT, "immunodbscan_gb300", "host"),
                    os.path.join(ROOT, "immunodbscan_gb300", "host", "psdbscan.cpp"), "-o",
                    str(d / "psdbscan"), "-L" + str(d), "-limmunodbscan_gb300", "-Wl,-rpath,$ORIGIN"],
                   check=True)
    w = synth.workload(0, scale=0.02)
    cf, inp, keep = _write_inputs(tmp_path, w, True, False)
    base = cf.read_text()
    cf.write_text(base + "\ncandidate_pairs buckets\n")
    r = subprocess.run([str(d / "psdbscan"), "--config_file", str(cf), "--input", str(inp)],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    lines = (tmp_path / "output_repertoire.csv").read_text().split("\n")
    copies = lines[0].split("\t").index("Copies")
    assert len(lines) > 3 and all(l.split("\t")[copies] == "7" for l in lines[1:-1])
    cf.write_text(base + "\ncandidate_pairs sideways\n")
    r = subprocess.run([str(d / "psdbscan"), "--config_file", str(cf), "--input", str(inp)],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode != 0
    assert "candidate_pairs must be auto or buckets" in (r.stdout + r.stderr)
