"""The opt-in forms of the build give the default form's trees: radix-sort tiles staged by bulk
copies (OTG_SORT_STAGE=1), the chunked persistent sort passes (OTG_SORT=chunked), and codegen
tiles staged by bulk copies (OTG_CODEGEN_STAGE=1). The switches are read once per process, so each
form builds in a child process, which prints a digest of its location keys and of its nodes in
canonical order (node order follows the emission's scheduling)."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import hashlib, sys
import numpy as np
import octree_gb300 as otg
rng = np.random.default_rng(31)
pts = rng.random((300_001, 3))
pts[:5000] = pts[7]
boxes = np.concatenate([pts[:100_000] - 0.001, pts[:100_000] + 0.002], 1)
out = []
for kind, ent, depth in (("points", pts, 10), ("points", pts[:4097], 9), ("boxes", boxes, 8)):
    t = otg.Tree(kind).create(ent, max_depth=depth, max_elements=12)
    h = hashlib.sha256(np.ascontiguousarray(t.location_keys()).tobytes())
    g = t.nodes()  # nodes in emission order: canonical form by key, entity ids ascending per node
    order = np.argsort(g["keys"], kind="stable")
    eoff = g["eoff"].astype(np.int64)
    for a in (g["keys"][order], g["min"][order], g["size"][order]):
        h.update(np.ascontiguousarray(a).tobytes())
    for i in order:
        h.update(np.sort(g["eids"][eoff[i] : eoff[i + 1]]).tobytes())
    out.append(h.hexdigest())
print(" ".join(out))
"""


def _digests(env_extra):
    env = dict(os.environ)
    env.pop("OTG_SORT", None)
    env.pop("OTG_SORT_STAGE", None)
    env.pop("OTG_CODEGEN_STAGE", None)
    env.update(env_extra)
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    p = subprocess.run([sys.executable, "-c", CHILD], env=env, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return p.stdout.split()


@pytest.mark.parametrize("variant", [{"OTG_SORT_STAGE": "1"}, {"OTG_SORT": "chunked"}, {"OTG_CODEGEN_STAGE": "1"}])
def test_build_variant_builds_the_same_trees(variant):
    assert _digests(variant) == _digests({})
