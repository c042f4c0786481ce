"""The golden step vectors of tests/golden/ (written by
tests/golden/make_golden.py from the oracle).

Counters, pair lists, contact body indices and row kinds must match exactly.
Floating-point values must match bit for bit on the architecture that wrote
the vectors (the manifest records it) and within 1e-12 relative on others:
x86-64 and aarch64 builds of the oracle were seen to differ in the last bit
of two solver multipliers of the grid case, and the GPU follows the oracle of
the machine it runs on bit for bit.  1e-12 is far inside the 1e-9 per-step
gate."""
import json
import os
import platform

import numpy as np
import pytest

from cannon_physics_gb300 import engine
from oracle import oracle_py as O
from tests.golden.make_golden import BODY_FIELDS, CASES

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = [c[0] for c in CASES]


def load(name):
    with np.load(os.path.join(HERE, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def case(name):
    return next(c for c in CASES if c[0] == name)


with open(os.path.join(HERE, "manifest.json")) as _f:
    MANIFEST = json.load(_f)
SAME_MACHINE = MANIFEST["machine"] == platform.machine()


def test_manifest_lists_every_case():
    assert sorted(MANIFEST["cases"]) == sorted(NAMES)


def _same_floats(a, b, what):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, what
    if SAME_MACHINE:
        assert a.tobytes() == b.tobytes(), what
    else:
        af, bf = a.astype(np.float64), b.astype(np.float64)
        assert np.all(np.abs(af - bf) <= 1e-12 * np.maximum(np.abs(bf), 1e-300) + (af == bf)), what


def _check(gold, bodies, counters, pairs, contacts, rows):
    assert np.array_equal(counters, gold["counters"])
    for f in BODY_FIELDS:
        if f == "sleep_state":
            assert np.array_equal(bodies[f], gold[f"body_{f}"])
        else:
            _same_floats(bodies[f], gold[f"body_{f}"], f)
    assert np.array_equal(pairs[0], gold["pair_a"]) and np.array_equal(pairs[1], gold["pair_b"])
    assert np.array_equal(np.stack([contacts["bi"], contacts["bj"]], 1).reshape(-1, 2), gold["contact_bodies"])
    _same_floats(contacts["ni"], gold["contact_ni"], "contact normals")
    _same_floats(rows["lambda_"], gold["row_lambda"], "row lambdas")
    assert np.array_equal(rows["kind"], gold["row_kind"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    _, make, steps = case(name)
    gold = load(name)
    sc = O.setup_scene(make())
    w = O.OracleWorld(sc)
    counters = np.zeros((steps, 4), np.int32)
    for s in range(steps):
        w.step(sc.dt, 1)
        inf = w.info()
        counters[s] = (inf.num_pairs, inf.num_contacts, inf.num_rows, inf.iterations)
    _check(gold, w.bodies(), counters, w.pairs(), w.contacts(), w.rows())


@pytest.fixture(scope="module")
def ctx():
    c = engine.Context(device=0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(ctx, name):
    _, make, steps = case(name)
    gold = load(name)
    sc = engine.setup_scene(make())
    w = ctx.world(sc)
    counters = np.zeros((steps, 4), np.int32)
    for s in range(steps):
        w.step(sc.dt, 1)
        inf = w.info()
        counters[s] = (inf.num_pairs, inf.num_contacts, inf.num_rows, inf.iterations)
    _check(gold, w.bodies(), counters, w.pairs(), w.contacts(), w.rows())
    w.destroy()
