"""The arrangement generators' oracle against the reference's own
src/pbf/util/pbf_arrangement.h (golden points made by
tests/golden/make_arrangement_golden.py), and the library's host-side
point counts.  No GPU needed."""
import ast
import os

import numpy as np
import pytest

from oracle import arrangement as A
from ssf_pbf_cuda_gb300 import api

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "arrangements", "points.npz")


def golden_cases():
    fx = np.load(GOLDEN)
    n = len([k for k in fx.files if k.endswith("_kind")])
    return [(str(fx[f"case{k}_kind"]), ast.literal_eval(str(fx[f"case{k}_args"])), fx[f"case{k}_points"])
            for k in range(n)]


CASES = golden_cases()


def abi_arrangement(kind, kw):
    if kind in ("volume", "line"):
        return api.arrangement(kind, origin=kw["origin"], end=kw["end"], space=kw["space"])
    if kind == "rectangle":
        return api.arrangement(kind, axis=kw["axis"], axis_value=kw["axis_value"], origin=kw["origin2"],
                               end=kw["end2"], space=kw["space"])
    return api.arrangement(kind, axis=kw["axis"], axis_value=kw["axis_value"], origin=kw["origin2"],
                           radius=kw["radius"], height=kw["height"], space=kw["space"])


@pytest.mark.parametrize("k", range(len(CASES)))
def test_oracle_matches_reference_generators(k):
    kind, kw, ref = CASES[k]
    ours = A.generate(kind, **kw)
    assert ours.shape == ref.shape
    if kind == "cylinder":  # cos / sin: last-bit differences between math libraries
        np.testing.assert_allclose(ours, ref, rtol=0, atol=4e-7 * max(1.0, float(np.abs(ref).max(initial=1))))
    else:
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("k", range(len(CASES)))
def test_library_point_counts(lib, k):
    kind, kw, ref = CASES[k]
    assert api.arrangement_count(abi_arrangement(kind, kw)) == len(ref)


def test_invalid_arrangements_rejected(lib):
    from ssf_pbf_cuda_gb300._lib import PbfError
    with pytest.raises(PbfError):
        api.arrangement_count(api.arrangement("volume", origin=(0, 0, 0), end=(1, 1, 1), space=0.0))
    with pytest.raises(PbfError):
        api.arrangement_count(api.arrangement("line", origin=(1, 1, 1), end=(1, 1, 1), space=0.1))
    with pytest.raises(PbfError):
        api.arrangement_count(api.arrangement("cylinder", origin=(0, 0), radius=0.01, height=1.0, space=0.1))
