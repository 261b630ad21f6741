"""The benchmark's accounting on the CPU: the reference arm prints the JSON line the contract
asks for (run on a small grid), and the byte model behind ``roofline.achieved`` and the e2e
upload count agree with hand counts from the model's own description."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from models import MODELS

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from gprmax_gb300.model import build_grid  # noqa: E402


def _grid(name):
    return build_grid(MODELS[name].splitlines(True), messages=False)


def _slab_cells(G):
    t = G.pmlthickness
    return ((t['x0'] + t['xmax']) * G.ny * G.nz + (t['y0'] + t['ymax']) * G.nx * G.nz
            + (t['z0'] + t['zmax']) * G.nx * G.ny)


def _dispersive_cells(G):
    poles = {m.numID for m in G.materials if m.poles > 0}
    ids = G.ID[:3, :G.nx, :G.ny, :G.nz]
    return int(np.count_nonzero(np.isin(ids, list(poles)).any(axis=0)))


@pytest.mark.parametrize('name,state_bytes', [('fs_hori1', 0), ('debye1', 24), ('mixed', 48)])
def test_algorithmic_bytes_match_a_hand_count(name, state_bytes):
    """H: 36 B per cell without IDs (every material non-magnetic); E: 40 B per cell; 16 B per
    slab cell and CFS order in each; the pole state on dispersive cells, 24 B per pole as real
    parts (Debye only) or 48 B complex (Lorentz or Drude present)."""
    G = _grid(name)
    cells = G.nx * G.ny * G.nz
    pml = _slab_cells(G) * 16 * len(G.cfs)
    assert bench.slab_cells(G) == _slab_cells(G)
    h, e = bench.algorithmic_bytes(G)
    assert h == cells * 36 + pml
    disp = _dispersive_cells(G) * state_bytes * G.maxpoles if G.maxpoles else 0
    assert e == cells * 40 + pml + disp
    if G.maxpoles:
        assert _dispersive_cells(G) > 0


def test_upload_bytes_count_every_host_array():
    G = _grid('debye1')
    n = (G.nx + 1) * (G.ny + 1) * (G.nz + 1)
    nmat = len(G.materials)
    expect = (6 * n * 4 + nmat * 5 * 4 * 2 + nmat * 3 * G.maxpoles * 8
              + sum(8 * 4 * p.ERA.size for p in G.pmls) + G.iterations * 4)
    assert bench.upload_bytes(G) == expect


def test_measured_traffic_takes_the_full_size_capture_only_for_its_grid():
    full = bench._profile_value(bench.TRAFFIC_FULL, 'dram_bytes_per_launch')
    cells = int(bench._profile_value(bench.TRAFFIC_FULL, 'cells'))
    per_cell = bench._profile_value(bench.TRAFFIC_PROFILE, 'dram_bytes_per_cell')
    assert bench.measured_traffic(cells) == (int(full), 'ncu, full-size launch')
    b, src = bench.measured_traffic(1000)
    assert b == int(round(per_cell * 1000)) and 'scaled' in src
    # the staged E sweep's captures (the kernel the soil runs)
    full = bench._profile_value(bench.STAGED_TRAFFIC_FULL, 'dram_bytes_per_launch')
    cells = int(bench._profile_value(bench.STAGED_TRAFFIC_FULL, 'cells'))
    per_cell = bench._profile_value(bench.STAGED_TRAFFIC_PROFILE, 'dram_bytes_per_cell')
    assert bench.measured_traffic(cells, staged=True) == (int(full), 'ncu, full-size launch')
    b, src = bench.measured_traffic(1000, staged=True)
    assert b == int(round(per_cell * 1000)) and 'scaled' in src


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference',
                          '--steps', '2', '--warmup', '3', '--grid', '48', '48', '24'],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith('{')]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r['impl'] == 'reference' and r['metric'] == r['unit'] == 'Mcells/s'
    assert r['value'] > 0 and r['n_gpus'] == 1 and r['warmup'] >= 3 and r['steps'] >= 2
    assert r['higher_is_better'] is True and r['vs_baseline'] is None
    assert r['config']['grid'] == [48, 48, 24] and r['config']['cells'] == 48 * 48 * 24
    cb = r['cpu_baseline']
    assert cb['value'] == r['value'] and cb['kind'] in ('reference', 'port') and cb['cores'] >= 1
    assert r['e2e'] == {'value': r['value'], 'unit': 'Mcells/s', 'h2d_bytes_per_step': 0,
                        'd2h_bytes_per_step': 0}
    assert r['gpu_launches'] == 0
