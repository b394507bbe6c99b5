"""The serving loop's deadline admission rule (mpmgpu_server_admits), a pure
host function: a queued request is admitted while every running request of
its dimension keeps elapsed + steps_left x (a + b R) within k times its time
alone, s (a + b n); requests already past their bound do not block."""
import pytest

A, B, K = 0.1, 1e-6, 4.0  # ms per step: a + b x resident particles


def admits(running, n, steps=100, waited=0.0, a=A, b=B, k=K):
    from nairn_gb300.gpu import server_admits
    return server_admits(a, b, k, running, n, steps, waited)


def test_an_idle_batch_admits_anything(gpu_lib):
    assert admits([], 50_000_000) == 1


def test_bound_of_a_running_request(gpu_lib):
    # 1e5 particles, 200 steps: 40 ms alone, bound 160 ms; half done in 20 ms
    r = [(100_000, 100, 200, 20.0)]
    assert admits(r, 1_000_000) == 1   # 20 + 100 x 1.2 = 140 <= 160
    assert admits(r, 2_000_000) == 0   # 20 + 100 x 2.2 = 240 > 160
    # the bound is exactly the line between them
    n_max = ((160.0 - 20.0) / 100 - A) / B - 100_000
    assert admits(r, int(n_max) - 1000) == 1 and admits(r, int(n_max) + 1000) == 0


def test_late_requests_do_not_block(gpu_lib):
    late = (100_000, 100, 200, 1000.0)      # already past 160 ms
    on_time = (100_000, 100, 200, 20.0)
    assert admits([late], 5_000_000) == 1
    assert admits([late, on_time], 5_000_000) == 0
    assert admits([late, on_time], 500_000) == 1


def test_every_running_request_is_checked(gpu_lib):
    big = (2_000_000, 500, 1000, 100.0)     # alone 2,100 ms: loose
    small = (20_000, 190, 200, 5.0)         # alone 24 ms, bound 96 ms
    # resident 2.02 M: the small run is late already (5 + 190 x 2.12 > 96) and does not block
    assert admits([big, small], 1_000_000) == 1
    tight = (20_000, 10, 200, 20.0)         # 20 + 10 x 2.12 = 41 <= 96: on time
    assert admits([big, tight], 1_000_000) == 1   # 20 + 10 x 3.12 = 51 still <= 96
    assert admits([big, tight], 8_000_000) == 0   # 20 + 10 x 10.12 = 121 > 96
    # (the big run would still be on time: 100 + 500 x 10.12 = 5,160 <= 8,400)


@pytest.mark.parametrize("bad", [dict(a=-1.0), dict(b=-1e-9), dict(k=0.5), dict(n=0), dict(steps=0),
                                 dict(waited=-1.0)])
def test_bad_arguments_are_refused(bad, gpu_lib):
    kw = dict(running=[(1000, 10, 20, 1.0)], n=1000)
    kw.update(bad)
    assert admits(**kw) == -1
