"""Failure paths of the device code, exercised without faulting a GPU.

The reference exits the process on any CUDA error (src/device/DevUtils.cu:12-22);
this library returns a status instead. The debug hooks of the C ABI make the
library take the same paths that a real failure takes:

* a bounded mbarrier wait made to run out on a barrier that nothing completes
  (no copy and no MMA in flight) sets the timeout bit: DR_ERR_TIMEOUT, then the
  context works on;
* a lower cap on the 8-wide traversal stack makes deep rays stop with the
  overflow bit: DR_ERR_STACK_OVERFLOW, for the public traversal and for the
  renderer, then the same scene traces bit-exact again;
* the n-th device allocation of a call made to fail: every allocation of
  scene creation, rendering, framebuffers, guiding networks and batches
  returns DR_ERR_OUT_OF_MEMORY, leaks no device memory, and leaves the
  context usable.
"""
from __future__ import annotations

import numpy as np
import pytest

from devilray_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _trace(native, scene, rays):
    d = torch.from_numpy(rays).cuda()
    hits = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
    scene.trace_closest(d, len(rays), hits)
    torch.cuda.synchronize()
    h = hits.cpu().numpy()
    return h[:, 0].copy().view(np.float32), h[:, 1].copy()


def _status_of(fn):
    try:
        fn()
    except Exception as e:  # noqa: BLE001 - the status is what is checked
        return getattr(e, "status", None)
    return 0


def test_expired_wait_reports_timeout(native, oracle):
    lib = native.load()
    c = native.Context(0)
    native.check(lib.dr_debug_expire_wait(c.handle, 1024, None))
    assert _status_of(c.check) == 5  # DR_ERR_TIMEOUT
    assert _status_of(c.check) == 0  # the check cleared the bit
    # a limit of no polls at all gives up at once
    native.check(lib.dr_debug_expire_wait(c.handle, 0, None))
    assert _status_of(c.check) == 5
    # the context goes on tracing, bit-exact
    half = scenes.density_half(4096)
    soup, _, _ = scenes.incoherent_soup(4096, seed=3, half=half)
    rays = scenes.incoherent_rays(20000, seed=4, half=half)
    scene = native.Scene(c, soup)
    t, prim = _trace(native, scene, rays)
    tc, pc = oracle.BBH(soup).trace_canonical(rays, slack=scene.info().slack)
    assert np.array_equal(_bits(t), _bits(tc)) and np.array_equal(prim, pc)
    assert _status_of(c.check) == 0


def test_stack_cap_reports_overflow(native, oracle):
    lib = native.load()
    c = native.Context(0)
    half = scenes.density_half(65536)
    soup, _, _ = scenes.incoherent_soup(65536, seed=5, half=half)
    rays = scenes.incoherent_rays(50000, seed=6, half=half)
    scene = native.Scene(c, soup)
    assert scene.info().layout == 8 and scene.info().depth >= 3
    native.check(lib.dr_debug_stack_limit(c.handle, 1))
    _trace(native, scene, rays)
    assert _status_of(c.check) == 6  # DR_ERR_STACK_OVERFLOW
    # the renderer's traversal reports it too
    spec = scenes.many_light(6 * 1280, 40, seed=3, half=6.0)
    rscene = native.Scene.from_spec(c, spec)
    acc = torch.zeros((32 * 24, 4), dtype=torch.float32, device="cuda")
    rscene.render(scenes.outside_camera(32, 24, distance=20.0, half=6.0), acc, spp=2, max_depth=6)
    torch.cuda.synchronize()
    assert _status_of(c.check) == 6
    # the full stack again: exact results, no error
    native.check(lib.dr_debug_stack_limit(c.handle, 0))
    t, prim = _trace(native, scene, rays)
    tc, pc = oracle.BBH(soup).trace_canonical(rays, slack=scene.info().slack)
    assert np.array_equal(_bits(t), _bits(tc)) and np.array_equal(prim, pc)
    assert _status_of(c.check) == 0
    assert lib.dr_debug_stack_limit(c.handle, 65) == 1  # DR_ERR_INVALID_ARGUMENT


def _workload(native, ctx, spec, cam):
    """Scene creation, a render, a framebuffer, a guiding network and a batch:
    every call that allocates device memory."""
    scene = native.Scene.from_spec(ctx, spec)
    n = cam["width"] * cam["height"]
    acc = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    scene.render(cam, acc, spp=2, max_depth=6, seed=1)
    torch.cuda.synchronize()
    fb = native.Framebuffer(ctx, cam["width"], cam["height"])
    g = native.Guide(ctx, seed=1, half_extent=1.0)
    acc2 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    native.render_batch(ctx, [native.make_job(scene, cam, acc2, spp=1, max_depth=4)])
    torch.cuda.synchronize()
    g.close()
    fb.close()
    scene.close()
    return acc.cpu().numpy()


def test_failed_allocations_return_out_of_memory(native, ctx):
    lib = native.load()
    spec = scenes.box_room(sphere_level=1)
    cam = scenes.camera(16, 12)
    want = _workload(native, ctx, spec, cam)  # also grows the context's scratch
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for k in range(1, 200):
        native.check(lib.dr_debug_fail_allocation(k))
        try:
            _workload(native, ctx, spec, cam)
        except native.DrError as e:
            assert e.status == 3, e  # DR_ERR_OUT_OF_MEMORY
            failures += 1
            continue
        finally:
            native.check(lib.dr_debug_fail_allocation(0))
        break  # the k-th allocation was never reached: every one was made to fail
    else:
        pytest.fail("the workload kept failing")
    assert failures >= 10, failures
    torch.cuda.synchronize()
    assert _status_of(ctx.check) == 0
    got = _workload(native, ctx, spec, cam)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 16 << 20, f"{(free0 - free1) >> 20} MiB of device memory not returned"
