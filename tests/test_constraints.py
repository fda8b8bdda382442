"""The product's template compiler against the reference's log.totem dumps
(157 templates: the bundled fixture patterns, fixed shapes with distinct and
repeated labels, random templates)."""
import pytest

import pattenmatching_sharedmemory_gb300 as pm
from pattenmatching_sharedmemory_gb300 import templates as T
from tests import cases as C
from tests import pmtest

GOLD = pmtest.load_constraint_golden()


def _norm(text: str) -> str:
    return "\n".join(l.rstrip() for l in text.splitlines() if l.strip())


@pytest.mark.parametrize("entry", GOLD, ids=lambda e: e["case"]["name"])
def test_constraint_dump_matches_reference(entry):
    p = C.make_pattern(entry["case"])
    assert _norm(p.dump_constraints()) == entry["dump"]


def test_pattern_too_large_rejected():
    p = pm.Pattern.from_edges(65, [(i, i + 1) for i in range(64)], [0] * 65)
    with pytest.raises(pm.PmError) as e:
        p.dump_constraints()
    assert e.value.code == pm.PM_E_PATTERN_TOO_LARGE


def test_cycle_canonical_rotation():
    # cycle 3-1-2 in pattern ids must be rotated to start at the smallest id
    p = pm.Pattern.from_edges(4, [(3, 1), (1, 2), (2, 3), (0, 3)], [0, 1, 2, 3])
    dump = p.dump_constraints()
    assert "Vertex Index : 1 -> 2 -> 3 -> 1" in dump or "Vertex Index : 1 -> 3 -> 2 -> 1" in dump


def test_template_generator_deterministic():
    a = T.random_template(7, 0.5, T.zipf_weights(4, 1.0), seed=42)
    b = T.random_template(7, 0.5, T.zipf_weights(4, 1.0), seed=42)
    assert (a.offsets == b.offsets).all() and (a.adj == b.adj).all() and (a.labels == b.labels).all()
