"""GPU: the serving loop over a real batch pool. Scenes join and leave the running batch at different steps
(queueing behind a scene limit); each request's final state must be the state of the same scene stepped
alone for its rollout length, bit for bit."""
import numpy as np
import pytest

from pcisph_gb300 import Batch, Fluid, scenes, setup_scene
from pcisph_gb300.batch import memory_model
from pcisph_gb300.serve import Request, Server

pytestmark = pytest.mark.gpu


def _requests():
    out = []
    kinds = [lambda k: scenes.batch_drop(900 + 150 * k, d=0.01, seed=20 + k, name=f"drop{k}"),
             lambda k: scenes.batch_dam(600 + 200 * k, 0.7 + 0.2 * k, 1.3, d=0.01, seed=30 + k, name=f"dam{k}")]
    for k in range(7):
        out.append(Request(k, 0.0, kinds[k % 2](k), steps=3 + (5 * k) % 9))
    return out


def test_served_rollouts_match_scenes_alone():
    reqs = _requests()
    bpp, bps = memory_model()
    total = sum(r.particles for r in reqs)
    bt = Batch(0, max_particles=total, max_scenes=3)
    srv = Server(bt, budget_bytes=10**12, bytes_per_particle=bpp, bytes_per_scene=bps, max_particles=total,
                 max_scenes=3)
    rep = srv.run(reqs, realtime=False)
    assert len(rep.completions) == len(reqs) and rep.queued_at_end == 0
    assert max(c.queueing for c in rep.completions) > 0  # some requests waited for a slot
    for c in rep.completions:
        r = reqs[c.rid]
        f = Fluid(0)
        setup_scene(f, r.scene, kernel_variant=2)
        f.step(r.steps)
        np.testing.assert_array_equal(c.position, f.get_field("position"), err_msg=r.scene.name)
        np.testing.assert_array_equal(c.velocity, f.get_field("velocity"), err_msg=r.scene.name)
        assert c.iterations == f.stats().total_iterations
        f.close()
    assert bt.info()[:2] == (0, 0)
