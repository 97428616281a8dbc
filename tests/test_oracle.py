"""The CPU oracle pinned against the reference's own outputs (CPU only).

tests/golden/*.npz were produced by running the reference project's compiled
decoders (tests/golden/make_golden.py); the oracle must reproduce every path.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("variant", ["serial", "omp"])
def test_oracle_matches_reference_paths(name, variant):
    args, z = load_golden(name)
    out = orc.decode(*args, variant=variant, nthreads=2)
    np.testing.assert_array_equal(out["path"], z["path_cpp"])
    for other in ("path_omp", "path_cpp_fast", "path_py"):
        if other in z:
            np.testing.assert_array_equal(z[other], z["path_cpp"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_loglik_matches_segment_scorer(name):
    args, z = load_golden(name)
    out = orc.decode(*args, tables=True)
    N, tm, em, _, sp, dp, obs = args
    sc = orc.score_segments(N, tm, em, sp, dp, obs, out["path"], out["seg_start"])
    if np.isfinite(out["loglik"]):
        assert abs(sc - out["loglik"]) <= 1e-9 * abs(sc)
    # the loglik is the tail score of the first best final state
    assert out["loglik"] == out["tail"].max()


def test_oracle_serial_and_omp_tables_identical():
    args, _ = load_golden("syn_config0")
    a = orc.decode(*args, tables=True)
    b = orc.decode(*args, variant="omp", nthreads=4, tables=True)
    for k in ("delta", "tail", "psi_state", "psi_dur"):
        np.testing.assert_array_equal(a[k], b[k])


def test_oracle_fast_build_agrees_on_fixture():
    args, z = load_golden("syn_config0")
    out = orc.decode(*args, variant="omp", nthreads=2, fast=True)
    np.testing.assert_array_equal(out["path"], z["path_cpp"])


def test_oracle_rejects_short_and_out_of_range():
    args, _ = load_golden("syn_config0")
    N, tm, em, dl, sp, dp, obs = args
    with pytest.raises(ValueError, match="T < D"):
        orc.decode(N, tm, em, dl, sp, dp, obs[:50])
    bad = obs.copy()
    bad[7] = em.shape[0]
    with pytest.raises(ValueError, match="out of range"):
        orc.decode(N, tm, em, dl, sp, dp, bad)


def test_reference_module_agrees_when_built():
    ref = orc.reference_module("ieee")
    if ref is None:
        pytest.skip("reference _native not built on this host (oracle/build_ref.sh)")
    import tensor_viterbi.synthetic as syn
    for seed in range(3):
        p = syn.discrete_problem(6, 30, 300, 8, 3.0, 20.0, seed=100 + seed)
        np.testing.assert_array_equal(orc.decode(*p.args())["path"], ref.decode_tensor_viterbi_cpp(*p.args()))
