"""Batched evaluation, CUDA-graph replay, device-resident MD and the serving loop on the GPU.

Batches: every structure's energy, forces and virial must be bit-identical to
evaluating it alone (per-structure arithmetic does not depend on its batch position).
MD: velocity Verlet as DynamicalSystem advance_verlet1/2; the skin-reuse path
(connection_calc_dists) must agree with rebuilding the list every step, and the
trajectory with a host loop of single evaluations.
"""
import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import models

from helpers import si_model, sic_model

pytestmark = pytest.mark.gpu


def _pot(path, precision="fp64"):
    from quip_gb300.potential import Potential
    return Potential(param_filename=path, precision=precision)


@pytest.fixture(scope="module")
def sic_gap(tmp_path_factory):
    return sic_model(tmp_path_factory.mktemp("sic_batch"))


@pytest.fixture(scope="module")
def si_gap(tmp_path_factory):
    return si_model(tmp_path_factory.mktemp("si_md"), M=200)


def _structures():
    rng = np.random.default_rng(21)
    s = [models.random_triclinic(int(k), rng=rng) for k in (9, 40, 130, 17, 75)]
    s.insert(2, models.si_primitive(rattle=0.03, seed=4))   # cutoff larger than the cell
    return s


@pytest.mark.parametrize("prec", ["fp64", "bf16x3", "tf32", "fp16"])
def test_batch_is_bit_identical_to_single(sic_gap, prec):
    pot = _pot(sic_gap, prec)
    structs = _structures()
    batch = pot.calc_batch(structs)
    for at, b in zip(structs, batch):
        a = pot.calc(at)
        assert a["energy"] == b["energy"]
        assert np.array_equal(a["force"], b["force"])
        assert np.array_equal(a["virial"], b["virial"])


def test_batch_with_an_empty_structure(sic_gap):
    pot = _pot(sic_gap)
    structs = _structures()[:3]
    empty = models.Atoms(np.zeros(0, np.int32), np.zeros((0, 3)), lattice=np.eye(3) * 6.0, pbc=True)
    res = pot.calc_batch(structs[:1] + [empty] + structs[1:])
    assert res[1]["energy"] == 0.0 and res[1]["force"].shape == (0, 3)
    assert res[0]["energy"] == pot.calc(structs[0])["energy"]
    assert res[2]["energy"] == pot.calc(structs[1])["energy"]


@pytest.mark.parametrize("prec", ["fp64", "tf32"])
def test_graph_replay_matches_direct_launches(sic_gap, prec):
    pot = _pot(sic_gap, prec)
    at = models.random_triclinic(120, rng=np.random.default_rng(5))
    ref = pot.calc(at)
    pot.set_option("graphs", 1)
    for _ in range(4):   # direct, capture, replay, replay
        r = pot.calc(at)
        assert r["energy"] == ref["energy"]
        assert np.array_equal(r["force"], ref["force"])
        assert np.array_equal(r["virial"], ref["virial"])
    moved = at.copy()
    moved.positions[7] += np.array([0.03, -0.02, 0.01])
    assert pot.calc(moved)["energy"] != ref["energy"]   # new positions are evaluated, not a stale replay


def _replicas(k, seed):
    return [models.si_diamond(2, rattle=0.05, seed=seed + i) for i in range(k)]


def test_md_conserves_energy(si_gap):
    from quip_gb300.md import MDReplicas
    pot = _pot(si_gap)
    md = MDReplicas(pot, _replicas(2, 30), dt=0.5, skin=0.5, temperature=300.0, seed=1)
    s0 = md.state()
    e0 = s0["energy"] + s0["kinetic"]
    md.step(60)
    s1 = md.state()
    e1 = s1["energy"] + s1["kinetic"]
    drift = np.abs(e1 - e0) / 64
    assert np.all(drift < 2e-4), drift
    assert md.counters()["steps"] == 60


def test_md_skin_reuse_agrees_with_rebuild_every_step(si_gap):
    from quip_gb300.md import MDReplicas
    pot = _pot(si_gap)
    reps = _replicas(2, 40)
    a = MDReplicas(pot, reps, dt=1.0, skin=0.5, temperature=1000.0, seed=3)
    b = MDReplicas(pot, reps, dt=1.0, skin=0.0, temperature=1000.0, seed=3)
    a.step(40)
    b.step(40)
    sa, sb = a.state(), b.state()
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-8
    assert np.abs(sa["energy"] - sb["energy"]).max() < 1e-8
    ca, cb = a.counters(), b.counters()
    assert cb["rebuilds"] == 41                     # every step plus the initial build
    assert 1 <= ca["rebuilds"] < 41                 # kept lists between rebuilds
    assert ca["graph_replays"] > 0


def test_md_kept_list_and_forces_match_oracle(si_gap):
    """Skin reuse against the oracle (connection_calc_dists, Connection.f95:1321-1445, under
    the skin rule :1086-1125): step until the list has been rebuilt at least once after the
    first build and the last step kept it (a refresh), then compare the refreshed list's
    pairs inside the cutoff -- (i, j, shift) and r -- with the oracle's neighbour list of the
    current positions, and the forces and energies with oracle calculations on those
    positions."""
    from quip_gb300.md import MDReplicas
    pot = _pot(si_gap)
    md = MDReplicas(pot, _replicas(2, 60), dt=1.0, skin=0.5, temperature=1000.0, seed=5)
    kept = False
    for step in range(1, 400):
        before = md.counters()["rebuilds"]
        md.step(1)
        kept = md.counters()["rebuilds"] == before
        if kept and md.counters()["rebuilds"] >= 2:
            break
    assert kept and md.counters()["rebuilds"] >= 2, md.counters()
    s = md.state()
    off, j, sh, r = md.neighbours()
    rc = pot.cutoff()
    om = oracle.OracleModel.from_xml(si_gap)
    for k, at in enumerate(_replicas(2, 60)):
        a0, a1 = s["offsets"][k], s["offsets"][k + 1]
        pos = s["pos"][a0:a1]
        o_off, o_j, o_sh, _, o_r = oracle.neighbours(pos, at.lattice, [1, 1, 1], rc)
        for a in range(a1 - a0):
            got = {(int(j[p]) - a0,) + tuple(sh[p]): r[p] for p in range(off[a0 + a], off[a0 + a + 1]) if r[p] < rc}
            ref = {(int(o_j[p]),) + tuple(o_sh[p]): o_r[p] for p in range(o_off[a], o_off[a + 1])}
            assert got.keys() == ref.keys()
            assert max(abs(got[t] - ref[t]) for t in ref) < 1e-12
        o = om.calc(pos, at.numbers, at.lattice, [1, 1, 1])
        assert np.abs(s["force"][a0:a1] - o["force"]).max() < 1e-7
        assert abs(s["energy"][k] - o["energy"]) / len(at) < 1e-8


def test_md_matches_host_verlet_loop(si_gap):
    """Five steps of the device integrator against velocity Verlet written on the host
    around single evaluations."""
    from quip_gb300.md import MDReplicas, masses, maxwell_boltzmann
    pot = _pot(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=50)
    v = maxwell_boltzmann(at.numbers, 800.0, seed=9)
    at.arrays["velo"] = v
    md = MDReplicas(pot, [at], dt=1.0, skin=0.3)
    md.step(5)
    s = md.state()
    m = masses(at.numbers)[:, None]
    x, vv = at.positions.copy(), v.copy()
    f = pot.calc(at)["force"]
    for _ in range(5):
        vv += 0.5 * 1.0 * f / m
        x += 1.0 * vv
        cur = at.copy()
        cur.positions = x
        f = pot.calc(cur)["force"]
        vv += 0.5 * 1.0 * f / m
    assert np.abs(s["pos"] - x).max() < 1e-10
    assert np.abs(s["velo"] - vv).max() < 1e-10


def test_serving_results_are_the_same_alone_and_in_the_mix(sic_gap):
    from quip_gb300.md import MDReplicas
    from quip_gb300.serving import Server, poisson_arrivals
    rng = np.random.default_rng(8)
    structs = [models.random_triclinic(int(k), rng=rng) for k in rng.integers(16, 160, 14)]
    # two bursts, the second while the first is being served
    arrivals = np.concatenate([poisson_arrivals(1e5, 7, seed=2), 0.05 + poisson_arrivals(1e5, 7, seed=3)])
    md = MDReplicas(_pot(sic_gap, "tf32"), _replicas(2, 60), dt=1.0, skin=0.5, temperature=1000.0, seed=4)
    srv = Server(sic_gap, precision="tf32", workers=2, budget_bytes=1 << 30, md=md)
    reqs, stats = srv.run(structs, arrivals)
    assert stats["requests"] == len(structs)
    assert stats["batches"] < len(structs)          # requests were batched together
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    alone = _pot(sic_gap, "tf32")
    alone.set_option("pairs", 0)   # the server's contexts run single-CTA GEMM tiles
    for r in reqs:
        a = alone.calc(r.atoms)
        assert abs(a["energy"] - r.result["energy"]) <= 1e-12 * max(1.0, abs(a["energy"]))
        assert np.abs(a["force"] - r.result["force"]).max() <= 1e-12


def test_serving_isolates_a_bad_request(sic_gap):
    """A request the library rejects (two atoms on top of each other) fails alone with
    its error; every other request of the same batch is served."""
    from quip_gb300.serving import Server
    rng = np.random.default_rng(12)
    structs = [models.random_triclinic(int(k), rng=rng) for k in (30, 50, 40)]
    bad = structs[1].copy()
    bad.positions[3] = bad.positions[0]
    structs[1] = bad
    srv = Server(sic_gap, precision="fp64", workers=1, budget_bytes=1 << 30)
    reqs, stats = srv.run(structs, np.zeros(len(structs)))
    assert "overlap" in reqs[1].result["error"]
    assert stats["failed"] == 1 and stats["requests"] == 2
    alone = _pot(sic_gap)
    for k in (0, 2):
        assert reqs[k].result["energy"] == alone.calc(structs[k])["energy"]


def test_bounded_device_wait_reports_timeout_and_context_survives(sic_gap):
    """Failure detection without a fault: a kernel waits on a barrier nothing signals;
    the wait gives up after its time bound (20 ms here, measured on the GPU's clock), the
    host reads GAPGPU_ERR_TIMEOUT well within a second, and the same context then
    evaluates normally."""
    import time
    from quip_gb300 import _lib
    pot = _pot(sic_gap, "tf32")
    at = models.random_triclinic(40, rng=np.random.default_rng(3))
    ref = pot.calc(at)["energy"]
    t0 = time.perf_counter()
    rc = pot._L.gapgpu_selftest_bounded_wait(pot._ctx, 20000)
    took = time.perf_counter() - t0
    assert rc == _lib.ERR_TIMEOUT
    assert 0.015 < took < 1.0, took
    assert b"bounded device-side" in pot._L.gapgpu_last_error()
    assert pot.calc(at)["energy"] == ref

