"""The drop-in executable (mantiis_gb300/bin/mantiis) with the reference's
argument interface and file layout (include/mantiisApp.hpp:131-142, 398-428):
inputs pore.dat / Kn.dat / localporesize.dat (column-major), outputs
ux.txt uy.txt rho.txt f.txt convergence.txt SimulationDetails.txt in the input
folder and reconstructed.dat in the working directory, compared with the
reference's gold files (test/run_tests.sh cases, 64x64, 100 steps)."""
import subprocess

import numpy as np
import pytest
from conftest import ROOT

BIN = ROOT / "mantiis_gb300" / "bin" / "mantiis"


def write_inputs(folder, fx):
    # the reference reads N*N numbers per file, x-major (column-major of [y, x])
    np.savetxt(folder / "pore.dat", np.asarray(fx["pore"]).T.reshape(-1), fmt="%d")
    np.savetxt(folder / "Kn.dat", np.asarray(fx["kn"]).T.reshape(-1), fmt="%.17g")
    np.savetxt(folder / "localporesize.dat", np.asarray(fx["locpore"]).T.reshape(-1), fmt="%.17g")


def test_usage_and_exit_code():
    # fewer than 6 arguments: usage on stderr, exit code 1 (include/mantiisApp.hpp:131-135)
    r = subprocess.run([str(BIN), "1", "False"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Usage:" in r.stderr and "<input_folder/>" in r.stderr


def test_missing_input_folder(tmp_path):
    r = subprocess.run([str(BIN), "1", "False", "64", str(tmp_path / "absent") + "/", "10"], capture_output=True,
                       text=True, timeout=120, cwd=tmp_path)
    assert r.returncode != 0


@pytest.mark.gpu
@pytest.mark.parametrize("case,preset", [("transport", "transport_test"), ("adsorption", "adsorption_test")])
def test_executable_matches_gold(tmp_path, fixture64, case, preset):
    folder = tmp_path / "io"
    folder.mkdir()
    write_inputs(folder, fixture64)
    r = subprocess.run([str(BIN), "1", "False", "64", str(folder) + "/", "100", "--preset", preset],
                       capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    ux = np.loadtxt(folder / "ux.txt").reshape(64, 64)
    uy = np.loadtxt(folder / "uy.txt").reshape(64, 64)
    rho = np.loadtxt(folder / "rho.txt").reshape(64, 64)
    umax = np.abs(fixture64[f"{case}_ux"]).max()
    e_ux = np.abs(ux - fixture64[f"{case}_ux"]).max() / umax
    e_uy = np.abs(uy - fixture64[f"{case}_uy"]).max() / umax
    e_rho = np.abs(rho - fixture64[f"{case}_rho"]).max() / np.abs(fixture64[f"{case}_rho"]).max()
    # the same bounds as the library-level gold tests (the text files carry
    # %.15g, far below these)
    if case == "transport":
        assert e_ux < 4e-6 and e_uy < 3e-6 and e_rho < 1e-11
    else:
        assert e_ux < 1e-5 and e_uy < 2.5e-5 and e_rho < 1.5e-5
    assert len(np.loadtxt(folder / "convergence.txt")) == 100
    assert np.loadtxt(folder / "f.txt").size == 64 * 64 * 9
    assert (folder / "SimulationDetails.txt").read_text().count("\n") >= 4
    assert (tmp_path / "reconstructed.dat").exists()
    assert "Timestep:" in r.stdout


def run_exe(tmp_path, folder, steps, *extra, threads=1):
    r = subprocess.run([str(BIN), str(threads), "False", "64", str(folder) + "/", str(steps), "--preset",
                        "transport_test", "--tol", "0", *extra], capture_output=True, text=True, timeout=600,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    return r


@pytest.mark.gpu
def test_binary_output_and_parallel_text(tmp_path, fixture64):
    one, many = tmp_path / "one", tmp_path / "many"
    for d in (one, many):
        d.mkdir()
        write_inputs(d, fixture64)
    run_exe(tmp_path, one, 30, "--output", "both", threads=1)
    run_exe(tmp_path, many, 30, "--output", "text", threads=8)
    # text formatted by 8 threads is byte-identical to 1 thread
    for name in ("f.txt", "ux.txt", "uy.txt", "rho.txt", "convergence.txt"):
        assert (one / name).read_bytes() == (many / name).read_bytes(), name
    # binary files hold the same values at full precision
    for name in ("ux", "uy", "rho", "f", "convergence"):
        b = np.fromfile(one / f"{name}.bin", dtype="<f8")
        t = np.loadtxt(one / f"{name}.txt").reshape(-1)
        assert b.size == t.size and np.allclose(b, t, rtol=1e-14, atol=0), name
    n_cells = int((np.asarray(fixture64["pore"]) == 1).sum())
    assert np.fromfile(one / "f_cells.bin", dtype="<f8").size == 9 * n_cells
    assert not (many / "f.bin").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("restart_file", ["f.txt", "f.bin", "f_cells.bin"])
def test_restart_continues_the_run(tmp_path, fixture64, restart_file):
    full, part = tmp_path / "full", tmp_path / "part"
    for d in (full, part):
        d.mkdir()
        write_inputs(d, fixture64)
    run_exe(tmp_path, full, 40, "--output", "binary")
    run_exe(tmp_path, part, 15, "--output", "both")
    saved = part / ("saved_" + restart_file)
    saved.write_bytes((part / restart_file).read_bytes())
    r = run_exe(tmp_path, part, 25, "--output", "binary", "--restart", str(saved), "--restart-step", "15")
    assert "Restarting from" in r.stdout
    assert "Number timesteps executed: 40" in (part / "SimulationDetails.txt").read_text()
    a = np.fromfile(full / "f_cells.bin", dtype="<f8")
    b = np.fromfile(part / "f_cells.bin", dtype="<f8")
    # FP64 files resolve the FP32 deviation state to ~1e-17, %.15g text to ~1e-16
    assert np.abs(a - b).max() < 1e-12
    conv_full = np.fromfile(full / "convergence.bin", dtype="<f8")
    conv_part = np.fromfile(part / "convergence.bin", dtype="<f8")
    assert conv_part.size == 25
    assert np.allclose(conv_part, conv_full[15:], rtol=1e-6, atol=0)
