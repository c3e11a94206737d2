"""The drop-in program's command line on a machine without a GPU: options
are checked before any device work, and a missing device is reported with
the reference's error exit (3) instead of a crash."""
import os
import subprocess

from conftest import PKG, has_gpu


def _run(built, tmp_path, args):
    exe = os.path.join(PKG, "edmd")
    return subprocess.run([exe] + args, cwd=tmp_path, capture_output=True, text=True, timeout=120)


def test_bad_engine_option_is_rejected(built, tmp_path):
    r = _run(built, tmp_path, ["--engine", "bogus"])
    assert r.returncode == 1
    assert "--engine auto|warp|round" in r.stderr


def test_missing_device_is_reported(built, tmp_path):
    if has_gpu():
        return
    r = _run(built, tmp_path, "--hex -N 64 --phi 0.5 -t 10 --quiet".split())
    assert r.returncode == 3
    assert "no CUDA device" in r.stderr
