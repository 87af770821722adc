"""Serving loop (nbpm_server_*): request validation and admission on the host, and on the GPU
the equality of a request's result alone, in a mix of other requests, and in a standalone run."""
import numpy as np
import pytest

from conftest import has_gpu
from nemaktis_gb300 import _lib, workloads


def small_request(Nx=24, Ny=20, Nz=6, nl=2, q=((0.0, 0.0), (0.05, 0.0)), seed=0, mask=False):
    js = workloads.settings_json((Nx, Ny, Nz), (0.25, 0.25, 0.25), list(np.linspace(0.5, 0.7, nl)), q,
                                 no="1.5", ne="1.7")
    lc = workloads.random_smooth((Nx, Ny, Nz), seed=seed)
    E = np.zeros((nl, len(q), 4, Ny, Nx), np.complex128)
    return js, lc, E


def test_submit_validates_on_the_host(lib):
    from nemaktis_gb300.serving import Server
    js, lc, E = small_request()
    with Server(hbm_budget_gb=1.0) as srv:
        with pytest.raises(_lib.NbpmError) as e:
            srv.submit("{not json", lc, E)
        assert e.value.code == 1
        with pytest.raises(_lib.NbpmError) as e:
            srv.submit(js, lc[:-3], E)
        assert e.value.code == 2 and "VectorField" in e.value.msg
        with pytest.raises(_lib.NbpmError) as e:
            srv.submit(js, lc, np.zeros(7, np.complex128))
        assert e.value.code == 2 and "OpticalFieldCollection" in e.value.msg
        assert srv.stats()["queued"] == 0


def test_request_above_budget_is_rejected(lib):
    from nemaktis_gb300.serving import Server
    js, lc, E = small_request(Nx=64, Ny=64, Nz=8, nl=4)
    with Server(hbm_budget_gb=1e-3) as srv:
        with pytest.raises(_lib.NbpmError) as e:
            srv.submit(js, lc, E)
        assert e.value.code == 5 and "budget" in e.value.msg


@pytest.mark.skipif(has_gpu(), reason="checks the no-device failure path")
def test_no_device_fails_loudly(lib):
    from nemaktis_gb300.serving import Server
    js, lc, E = small_request()
    with Server() as srv:
        r = srv.submit(js, lc, E)
        with pytest.raises(_lib.NbpmError) as e:
            r.wait(timeout=60)
        assert e.value.code == 4
        assert srv.stats()["failed"] == 1
    assert not E.any()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_alone_equals_mix_equals_standalone(gpu, precision):
    from nemaktis_gb300 import api
    from nemaktis_gb300.serving import Server
    js, lc, E_alone = small_request(Nx=32, Ny=28, Nz=9, nl=3, seed=1)
    E_mix = np.zeros_like(E_alone)
    E_plan = np.zeros_like(E_alone)
    api.run(js, lc, E_plan, precision=precision)
    with Server(precision=precision, slabs_per_round=3, round_voxel_steps=0) as srv:
        srv.submit(js, lc, E_alone).wait(timeout=300)
        others = [small_request(Nx=48, Ny=40, Nz=13, nl=2, seed=2), small_request(Nx=16, Ny=16, Nz=4, nl=1, seed=3,
                                                                                  q=((0.0, 0.0),)),
                  small_request(Nx=40, Ny=24, Nz=7, nl=4, seed=4)]
        reqs = [srv.submit(*others[0])]
        reqs.append(srv.submit(js, lc, E_mix))
        reqs += [srv.submit(*o) for o in others[1:]]
        for r in reqs:
            assert r.wait(timeout=300)["state"] == "done"
        st = srv.stats()
        assert st["done"] == 5 and st["failed"] == 0 and st["bytes_in_use"] == 0
    np.testing.assert_array_equal(E_alone, E_plan)
    np.testing.assert_array_equal(E_mix, E_plan)
    for js_o, lc_o, E_o in others:
        ref = np.zeros_like(E_o)
        api.run(js_o, lc_o, ref, precision=precision)
        np.testing.assert_array_equal(E_o, ref)


@pytest.mark.gpu
def test_round_quantum_does_not_change_results(gpu):
    from nemaktis_gb300.serving import Server
    js, lc, E1 = small_request(Nx=36, Ny=30, Nz=11, nl=3, seed=7)
    E2 = np.zeros_like(E1)
    with Server(round_voxel_steps=1.0) as srv:  # one slab per round
        srv.submit(js, lc, E1).wait(timeout=300)
    with Server(round_voxel_steps=1e12) as srv:  # every slab in one round
        srv.submit(js, lc, E2).wait(timeout=300)
    np.testing.assert_array_equal(E1, E2)


@pytest.mark.gpu
def test_budget_limits_requests_in_flight(gpu):
    from nemaktis_gb300.serving import Server
    reqs = [small_request(Nx=40, Ny=40, Nz=10, nl=3, seed=s) for s in range(4)]
    with Server(hbm_budget_gb=1.0) as srv:
        first = srv.submit(*reqs[0])
        need = first.poll()["device_bytes"]
    budget = 1.5 * need / 1e9  # room for one request at a time
    with Server(hbm_budget_gb=budget) as srv:
        hs = [srv.submit(*r) for r in reqs]
        for h in hs:
            assert h.wait(timeout=300)["state"] == "done"
        st = srv.stats()
        assert st["peak_bytes"] <= st["budget_bytes"]
        assert st["peak_bytes"] < 2 * need
    for js, lc, E in reqs:
        assert np.isfinite(E).all() and np.abs(E).max() > 0


@pytest.mark.gpu
def test_cancel(gpu):
    from nemaktis_gb300.serving import Server
    big = small_request(Nx=96, Ny=96, Nz=40, nl=4, seed=5)
    with Server(max_active=1) as srv:
        a = srv.submit(*big)
        b = srv.submit(*small_request(seed=6))
        b.cancel()
        a.cancel()
        sa, sb = a.wait(timeout=300)["state"], b.wait(timeout=300)["state"]
        assert sb == "cancelled"
        assert sa in ("cancelled", "done")
        assert srv.stats()["bytes_in_use"] == 0
