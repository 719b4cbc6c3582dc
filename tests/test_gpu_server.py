"""Event server (ccake_server_*): events of uneven sizes advanced concurrently
give the same states as the same events run one at a time; admission under
a tight device-memory budget; the freeze-out stop."""
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, ics

pytestmark = pytest.mark.gpu


def events(k=6):
    # small lattices (1-2 fm wide) hold mostly the 10 MeV/fm^3 floor, below
    # 150 MeV: a freeze-out temperature of 2 MeV keeps them running to tau_max
    out = []
    for j, side in enumerate([20, 28, 36, 44, 24, 32][:k]):
        p, rc = ics.hotspots_2d(n_side=side, n_hot=4, seed=100 + j)
        out.append((p, dataclasses.replace(rc, freeze_out_T=2.0 / 197.3269804)))
    return out


def standalone(p, rc, steps):
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    g.step(steps)
    return {f: g.get(f) for f in ("x", "u0", "ext_s", "T")}


@pytest.mark.parametrize("precision", [0, 1])
def test_concurrent_events_match_standalone_runs(precision):
    # FP64 events advance on streams of their own; mixed-form events are
    # advanced together by grouped launches (one launch of each step kernel
    # for every event). Either way each event's state is the same bits as
    # the event run alone.
    evs = [(p, dataclasses.replace(rc, precision=precision)) for p, rc in events()]
    steps = 30
    srv = api.Server(steps_per_launch=7)
    tickets = [srv.submit(p, rc, rc.t0 + steps * rc.dt) for p, rc in evs]
    srv.wait_all()
    for t, (p, rc) in zip(tickets, evs):
        r = srv.poll(t)
        assert r["state"] == "done", r
        assert r["steps"] == steps
        assert r["grouped"] == precision
        assert abs(r["tau"] - (rc.t0 + steps * rc.dt)) < 1e-9
        assert r["latency_s"] >= r["queue_s"] >= 0
        ref = standalone(p, rc, steps)
        for f, v in ref.items():
            assert np.array_equal(srv.get(t, f), v), f
        srv.release(t)
    srv.close()


def test_group_members_join_and_leave_between_periods():
    # mixed-form events with different lengths, some submitted while the
    # group runs: members leave the group at their own tau_max (the device
    # stops them before the step that would pass it) and newcomers join
    # between periods; every event still equals its standalone run bit for bit
    import time
    evs = [(p, dataclasses.replace(rc, precision=1)) for p, rc in events()]
    lengths = [7, 25, 40, 13, 31, 18]
    srv = api.Server()
    tickets = [srv.submit(p, rc, rc.t0 + k * rc.dt) for (p, rc), k in zip(evs[:3], lengths[:3])]
    time.sleep(0.05)
    tickets += [srv.submit(p, rc, rc.t0 + k * rc.dt) for (p, rc), k in zip(evs[3:], lengths[3:])]
    srv.wait_all()
    for t, (p, rc), k in zip(tickets, evs, lengths):
        r = srv.poll(t)
        assert r["state"] == "done" and r["grouped"] == 1 and r["steps"] == k, r
        ref = standalone(p, rc, k)
        for f, v in ref.items():
            assert np.array_equal(srv.get(t, f), v), (k, f)
        srv.release(t)
    srv.close()


def test_tight_budget_admits_one_event_at_a_time():
    # equal events and a budget that holds one of them, not two
    evs = [(p, dataclasses.replace(rc, freeze_out_T=2.0 / 197.3269804))
           for p, rc in (ics.hotspots_2d(n_side=30, n_hot=4, seed=300 + j) for j in range(4))]
    need = api.estimate_device_bytes(evs[0][1], evs[0][0].n)
    srv = api.Server(hbm_budget_bytes=int(1.5 * need), steps_per_launch=5)
    tickets = [srv.submit(p, rc, rc.t0 + 10 * rc.dt) for p, rc in evs]
    srv.wait_all()
    res = [srv.poll(t) for t in tickets]
    assert all(r["state"] == "done" and r["steps"] == 10 for r in res)
    # FIFO and sequential: each later event waited at least until the previous finished
    lat = [r["latency_s"] for r in res]
    q = [r["queue_s"] for r in res]
    for a in range(1, len(res)):
        assert q[a] >= q[a - 1]
    assert lat[-1] >= max(lat[:-1])
    srv.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_freeze_out_stops_an_event(precision):
    p, rc = events(1)[0]
    # 197 MeV: every particle starts below it and is frozen at initialisation.
    # A grouped (mixed-form) event is stopped by the device before its first
    # step, as the reference's loop tests continue_evolution before each step;
    # an event advanced alone is stopped after its first quantum.
    rc = dataclasses.replace(rc, freeze_out_T=1.0, particlization=1, precision=precision)
    srv = api.Server(steps_per_launch=5)
    t = srv.submit(p, rc, rc.t0 + 1000 * rc.dt)
    srv.wait_all()
    r = srv.poll(t)
    assert r["state"] == "done" and r["frozen"] == 1
    assert r["steps"] == (0 if precision else 5)
    srv.close()
