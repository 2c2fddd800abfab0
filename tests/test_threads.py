"""A context may be driven from any host thread: every entry point makes the context's device
current for the call and restores the caller's device afterwards. A context created on the main
thread is drawn from a worker thread (whose current device is whatever the runtime gives a new
thread, device 0) and must give the oracle's image; with two or more GPUs the context lives on
device 1, so a draw that ran on the thread's current device instead would fail or differ."""
import threading

import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from helpers import assert_outputs_match, render

pytestmark = pytest.mark.gpu


def _draw_on_worker(lib, device, scene):
    r = A.Renderer(lib, device)
    inst = S.SceneInstance(r, scene)
    out, errors = {}, []

    def work():
        try:
            inst.render()
            r.waitIdle()
            out["img"] = [inst.outputs()]
        except Exception as e:   # surfaced in the main thread below
            errors.append(e)

    t = threading.Thread(target=work)
    t.start()
    t.join()
    r.destroy()
    if errors:
        raise errors[0]
    return out["img"]


def _scene():
    return S.config_plain_small(width=320, height=240)


def test_context_drawn_from_a_worker_thread(cuda_lib, oracle_lib):
    scene = _scene()
    assert_outputs_match(_draw_on_worker(cuda_lib, 0, scene), render(oracle_lib, scene)[0], "worker thread")


def test_context_on_device_1_drawn_from_a_worker_thread(cuda_lib, oracle_lib):
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    scene = _scene()
    before = torch.cuda.current_device()
    img = _draw_on_worker(cuda_lib, 1, scene)
    assert torch.cuda.current_device() == before
    assert_outputs_match(img, render(oracle_lib, scene)[0], "device 1, worker thread")
