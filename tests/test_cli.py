"""speo_gpu: the reference driver's command line (src/main.cc flags) and record file
(Results/SPEO_GPU.csv, src/island_EA.cc:13-31, 146-171) over the library."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
CLI = REPO / "speo-gpu-single-control_gb300" / "lib" / "speo_gpu"
HEADER = ("function_ID,run_ID,dim,best_fitness,time_period,communication_percentage,total_FEs,node_num,GPU_num,"
          "island_num,total_pop_size,subisland_size,interval,migration_size,migration_rate,buffer_capacity,"
          "migration_topology,buffer_manage,regroup_option,configure_EA,EA_parameters")


def _cli():
    if not CLI.exists():
        from speo_gb300 import build

        build.build_cli()
    return CLI


@pytest.mark.parametrize("args", [["-dim", "0"], ["-configure_EA", "sometimes"], ["-total_functions", "5"],
                                  ["-regroup_option", "shuffle"], ["-buffer_capacity", "65"], ["-dim"],
                                  ["-island_size", "64", "-subisland_size", "128"],
                                  ["-island_size", "64", "-subisland_size", "2"]])
def test_cli_rejects_bad_flags_before_touching_the_gpu(tmp_path, args):
    res = subprocess.run([str(_cli()), *args], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert res.returncode == 2 and "speo_gpu:" in res.stderr
    assert not (tmp_path / "Results").exists()


def _write_instances(tmp_path, fids, D):
    from speo_gb300.instances import make_instance_multi, uses_shuffle, write_reference_data_multi

    for fid in fids:
        o, M, S = make_instance_multi(fid * 101 + D, D, fid)
        write_reference_data_multi(str(tmp_path), fid, o, M, S if uses_shuffle(fid) else None)


def _run(tmp_path, *args):
    res = subprocess.run([str(_cli()), *args], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    rows = (tmp_path / "Results" / "SPEO_GPU.csv").read_text().splitlines()
    return res.stdout, rows


@pytest.mark.gpu
def test_cli_runs_and_records_like_the_reference(tmp_path):
    _write_instances(tmp_path, [9, 23, 29], 10)
    args = ["-dim", "10", "-total_functions", "9-9", "-total_runs", "1-2", "-max_base_FEs", "3000", "-GPU_num", "3",
            "-island_size", "64", "-interval", "5", "-migration_size", "4", "-buffer_capacity", "8",
            "-regroup_option", "dynamic_and_random", "-subisland_size", "16"]
    out, rows = _run(tmp_path, *args)
    assert rows[0] == HEADER
    assert len(rows) == 3
    lines = [l for l in out.splitlines() if l.startswith("Run: ")]
    assert len(lines) == 2 and out.splitlines()[-1].startswith("Total Elapsed time: ")
    for run, row in zip((1, 2), rows[1:]):
        f = row.split(",")
        assert len(f) == 21
        assert f[:3] == ["9", str(run), "10"]
        assert float(f[3]) >= 0 and float(f[4]) > 0 and 0 <= float(f[5]) <= 1
        assert f[6:] == ["30000", "1", "3", "3", "192", "-1", "5", "4", "0.5", "8", "dynamicConnect", "DP",
                         "dynamic_and_random", "constant", "CR/F=0.9/0.5_rand/1/bin"]
    # deterministic: the same flags give the same best values
    other = tmp_path / "again"
    other.mkdir()
    _write_instances(other, [9], 10)
    _, rows2 = _run(other, *args)
    assert [r.split(",")[3] for r in rows2[1:]] == [r.split(",")[3] for r in rows[1:]]
    # composition / hybrid-composition functions, other buffer policies and regroup options
    _, rows3 = _run(tmp_path, "-dim", "10", "-total_functions", "23-23", "-total_runs", "1-1", "-max_base_FEs",
                    "2000", "-GPU_num", "2", "-island_size", "40", "-buffer_manage", "FIFO", "-regroup_option",
                    "static_and_random", "-configure_EA", "dynamic", "-subisland_size", "10")
    f = rows3[-1].split(",")
    assert f[0] == "23" and f[11] == "10" and f[17] == "FIFO" and np.isfinite(float(f[3]))
    _, rows4 = _run(tmp_path, "-dim", "10", "-total_functions", "29-29", "-total_runs", "3-3", "-max_base_FEs",
                    "1000", "-GPU_num", "1", "-island_size", "32", "-buffer_manage", "LIFO")
    f = rows4[-1].split(",")
    assert f[:2] == ["29", "3"] and f[8] == "1" and np.isfinite(float(f[3]))


@pytest.mark.gpu
def test_cli_reports_a_missing_instance(tmp_path):
    res = subprocess.run([str(_cli()), "-dim", "10", "-total_functions", "9-9", "-total_runs", "1-1"], cwd=tmp_path,
                         capture_output=True, text=True, timeout=120)
    assert res.returncode == 1 and "cannot read input_data" in res.stderr
