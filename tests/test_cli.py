"""The drop-in ClusterSM binary's command line and exit statuses (main.cu:26-34;
CLI11's RequiredError is 106, ExtrasError 109, ConversionError 105) on the
paths that end before the device is opened, plus the no-device status on a
host without a GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "clustersm_gb300" / "bin" / "ClusterSM"
EX = ROOT / "tests" / "golden" / "example"


def run(*args):
    assert CLI.exists(), "build the CLI first (__graft_entry__.build())"
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=120)


def test_help():
    r = run("--help")
    assert r.returncode == 0 and "-q <query graph path>" in r.stdout


@pytest.mark.parametrize("args,code", [
    ((), 106),
    (("-q", EX / "example_q_01.in"), 106),
    (("-d", EX / "example_g_01.in"), 106),
    (("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--bogus"), 109),
    (("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--gpu", "x"), 105),
    (("-q", EX / "example_q_01.in", "-d", EX / "example_g_01.in", "--gpu", "-1"), 105),
])
def test_option_errors(args, code):
    assert run(*args).returncode == code


def test_file_errors(tmp_path):
    missing = tmp_path / "missing.in"
    r = run("-q", missing, "-d", EX / "example_g_01.in")
    assert r.returncode == 2 and "reading the query graph" in r.stderr          # SMG_ERR_IO
    bad = tmp_path / "bad.in"
    bad.write_text("t 2 1\nv 0 0 1\nv 1 0 1\ne 0 5\n")
    r = run("-q", EX / "example_q_01.in", "-d", bad)
    assert r.returncode == 3 and "reading the data graph" in r.stderr          # SMG_ERR_FORMAT
    disc = tmp_path / "disconnected.in"
    disc.write_text("t 4 2\nv 0 0 1\nv 1 0 1\nv 2 0 1\nv 3 0 1\ne 0 1\ne 2 3\n")
    r = run("-q", disc, "-d", EX / "example_g_01.in")
    assert r.returncode == 4 and "preparing the query" in r.stderr             # SMG_ERR_QUERY


def test_equals_form_and_no_device():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    r = run(f"-q={EX / 'example_q_01.in'}", f"-d={EX / 'example_g_01.in'}", "--gpu=0")
    if has_gpu:
        assert r.returncode == 0 and r.stdout.strip().splitlines()[-1] == "num_res: 4"
    else:
        assert r.returncode == 9 and "opening the device" in r.stderr              # SMG_ERR_NO_DEVICE
