"""bench.py's ``gpu_launches`` claim, from its launch-count model of one
frequency-solve, against the ncu launch lists committed under profiles/
(6048-panel array, deep water, 30 modes, 8 headings): the captured launches
less the kernels that run once per mesh (named in each summary)."""
import importlib.util
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _captured(name):
    with open(os.path.join(ROOT, "profiles", name)) as f:
        m = re.search(r"Captured launches: (\d+)", f.read())
    assert m, name
    return int(m.group(1))


@pytest.mark.parametrize("profile,prec,once_per_mesh", [
    ("launches_mixed_step_6048.md", 1, 4),   # k_prep_panels, k_panel_gauss, k_mixed_near_list<1>, <0>
    ("launches_plain_step_6048.md", 0, 2),   # k_prep_panels, k_panel_gauss
])
def test_launch_model_matches_the_committed_launch_lists(bench, profile, prec, once_per_mesh):
    assert bench._launch_count(6048, prec, sweeps=1) == _captured(profile) - once_per_mesh
