"""CPU: the headless C++ runner builds against the library and handles its arguments without a GPU."""
import subprocess

from pcisph_gb300 import build


def test_runner_builds_and_prints_usage():
    exe = build.build_cli()
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "-i scene.xraw" in r.stdout


def test_runner_reports_a_missing_scene(tmp_path):
    exe = build.build_cli()
    r = subprocess.run([exe, "-i", str(tmp_path / "none.xraw")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "File not found" in r.stderr
    r = subprocess.run([exe, "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
