"""The `test` driver: the reference's command line, algorithm table and
output (Tridiagonal_CUDA/test.cpp:141-172, helpers.h:12-65)."""
import re
import subprocess

import pytest

from tests.conftest import ROOT

DRIVER = ROOT / "tridiagonalsolver_gb300" / "lib" / "test"
REF_FLOAT = ["cuSparse sgtsv", "Thomas", "CR", "shmem PCR-pThomas", "shmem PCR-half-pThomas", "reg PCR-pThomas",
             "reg PCR-half-pThomas", "shmem WM-pGE", "shmem WM-half-pGE", "reg WM-pGE", "reg WM-half-pGE",
             "reg-4 CR", "reg-8 CR", "reg-16 CR", "BPLG WM", "BPLG LF", "BPLG CR", "BPLG PCR"]


@pytest.fixture(scope="module")
def driver():
    from tridiagonalsolver_gb300 import build

    build.build()
    assert DRIVER.exists()
    return DRIVER


def test_usage_and_algorithm_table(driver):
    p = subprocess.run([str(driver)], capture_output=True, text=True)
    assert p.returncode == 1
    assert "USAGE:" in p.stdout and "<precision> <algorithm> <size> <batch> <repetitions>" in p.stdout
    single = p.stdout.split("single-precision algorithms:")[1].split("double-precision algorithms:")[0]
    names = re.findall(r"^\s*(\d+): (.+)$", single, flags=re.M)
    for i, nm in enumerate(REF_FLOAT):
        assert (str(i), nm) in names
    # names go into one CSV field
    for _, nm in re.findall(r"^\s*(\d+): (.+)$", p.stdout, flags=re.M):
        assert "," not in nm


@pytest.mark.parametrize("args", [["2", "1", "64", "4", "1"], ["0", "-1", "64", "4", "1"], ["0", "1", "0", "4", "1"],
                                  ["1", "1", "64", "0", "1"], ["1", "1", "64", "4", "0"]])
def test_invalid_arguments(driver, args):
    p = subprocess.run([str(driver), *args], capture_output=True, text=True)
    assert p.returncode == 1 and "USAGE:" in p.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("prec,algo,tol", [(1, a, 1e-12) for a in (0, 1, 2, 3, 5, 7, 9, 11, 13, 32, 33)] +
                         [(0, a, 2e-5) for a in (0, 1, 2, 4, 6, 8, 10, 12, 14, 15, 16, 17, 32, 33)])
def test_runs_and_reports(cuda, driver, tmp_path, prec, algo, tol):
    csv = tmp_path / "out.csv"
    p = subprocess.run([str(driver), str(prec), str(algo), "512", "96", "2", str(csv)], capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    mx = float(re.search(r"Max:\s+(\S+)", p.stdout).group(1))
    assert mx <= tol, p.stdout
    assert "Throughput:" in p.stdout and "condition number" in p.stdout
    row = csv.read_text().strip().split(",")
    assert len(row) == 11 and int(row[0]) == 512 and int(row[1]) == 96
