"""The autotuner's table file (BORA_TUNE_FILE) on the host: entries are read on first use,
malformed or out-of-range entries are skipped, and bora_flip_tune_table reports the table
(no GPU needed: reading the table launches nothing)."""
import os
import subprocess
import sys
import textwrap

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _table_in_subprocess(env):
    code = textwrap.dedent("""
        from vare_gb300 import flip
        for row in flip.tune_table():
            print(*row)
    """)
    out = subprocess.run([sys.executable, "-c", code], env=env, cwd=REPO, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return [tuple(line.split()) for line in out.stdout.splitlines() if line.strip()]


def test_table_file_is_loaded(tmp_path):
    lib = os.path.join(REPO, "vare_gb300", "_lib", "libbora_flip.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    path = tmp_path / "tune.txt"
    path.write_text("0 0 12 2 0.040\n"        # level 0, 8 tiles per block
                    "1 0 12 3 0.0147\n"       # level 1, 512 threads
                    "0 0 5 7 0.001\n"         # shape out of range: skipped
                    "9 0 5 0 0.001\n"         # unknown group: skipped
                    "5 0 9 0 0.002\n")        # level 2 of batches, 64 threads
    rows = _table_in_subprocess(dict(os.environ, BORA_TUNE_FILE=str(path)))
    got = {(int(g), int(d), int(c)): (int(v), float(m)) for g, d, c, v, m in rows}
    assert got == {(0, 0, 12): (2, 0.04), (1, 0, 12): (3, 0.0147), (5, 0, 9): (0, 0.002)}


def test_no_file_no_table():
    lib = os.path.join(REPO, "vare_gb300", "_lib", "libbora_flip.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    env = dict(os.environ)
    env.pop("BORA_TUNE_FILE", None)
    assert _table_in_subprocess(env) == []
