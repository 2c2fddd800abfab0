"""The neural IBL shader: Python face of the sglc_neural_* C ABI (include/softgl_cuda.h) and the
train / evaluate / fall-back pipeline around it.

A `NeuralShader` is a small MLP (12 inputs with a 6-frequency encoding, 2 x 64 ReLU, 3 outputs;
BF16 weights, FP32 accumulation on the tensor cores) that replaces the image-based-lighting term
of the PBR fragment shader (PbrSoft.h:291-309). `train_neural_ibl` renders training views with
the plain shader while capturing fragment records, trains the network on the GPU with the
library's own tensor-core forward / backward / Adam kernels, renders held-out views with both
shaders and keeps the network bound only if its PSNR against the plain shader reaches the
threshold (per material; otherwise the plain shader stays: the fallback).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import api as A
from . import scenes as S

RECORD_FLOATS = 16


class _TrainParams(C.Structure):
    _fields_ = [("steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("seed", C.c_uint64)]


_P = C.c_void_p
NEURAL_SIGS = {
    "neural_create": ([_P, C.c_uint64, C.POINTER(_P)], C.c_int32),
    "neural_destroy": ([_P], C.c_int32),
    "neural_param_count": ([], C.c_int64),
    "neural_set_params": ([_P, _P, C.c_int64], C.c_int32),
    "neural_get_params": ([_P, _P, C.c_int64], C.c_int32),
    "neural_set_records": ([_P, _P, C.c_int64], C.c_int32),
    "neural_get_records": ([_P, _P, C.c_int64, C.c_int64], C.c_int32),
    "neural_capture": ([_P, _P, C.c_int64, C.c_int32], C.c_int32),
    "neural_record_count": ([_P, C.POINTER(C.c_int64)], C.c_int32),
    "neural_train": ([_P, C.POINTER(_TrainParams), C.POINTER(C.c_float)], C.c_int32),
    "neural_gradients": ([_P, C.c_int64, C.c_int64, _P, C.POINTER(C.c_float)], C.c_int32),
    "neural_infer": ([_P, C.c_int64, C.c_int64, _P], C.c_int32),
    "program_set_neural_shader": ([_P, C.c_int32, _P], C.c_int32),
    "neural_set_test_flags": ([_P, C.c_int32], C.c_int32),
}
NEURAL_FUNCTIONS = tuple(NEURAL_SIGS)


def _bind(cdll: C.CDLL) -> Dict[str, object]:
    fns = {}
    for name, (args, res) in NEURAL_SIGS.items():
        f = getattr(cdll, "sglc_" + name)
        f.argtypes = args
        f.restype = res
        fns[name] = f
    return fns


class NeuralShader:
    """One network on a renderer's context (sglc_neural)."""

    def __init__(self, renderer: A.Renderer, seed: int = 1):
        self.r = renderer
        self.fn = _bind(renderer.lib.cdll)
        h = _P()
        self._check(self.fn["neural_create"](renderer.ctx, seed, C.byref(h)), "neural_create")
        self.h = h
        self.n_params = int(self.fn["neural_param_count"]())

    def _check(self, st: int, name: str) -> None:
        if st != 0:
            msg = self.r.lib.fn["last_error"](self.r.ctx)
            raise A.SoftGLError(st, "sglc_" + name, msg.decode() if msg else "")

    def destroy(self) -> None:
        if self.h:
            self.fn["neural_destroy"](self.h)
            self.h = None

    # -- parameters and records
    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(self.fn["neural_get_params"](self.h, out.ctypes.data, out.size), "neural_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.fn["neural_set_params"](self.h, p.ctypes.data, p.size), "neural_set_params")

    def set_records(self, rec: np.ndarray) -> None:
        rec = np.ascontiguousarray(rec, dtype=np.float32).reshape(-1, RECORD_FLOATS)
        self._check(self.fn["neural_set_records"](self.h, rec.ctypes.data, rec.shape[0]), "neural_set_records")

    def get_records(self, first: int = 0, count: Optional[int] = None) -> np.ndarray:
        if count is None:
            count = self.record_count() - first
        out = np.zeros((count, RECORD_FLOATS), np.float32)
        self._check(self.fn["neural_get_records"](self.h, out.ctypes.data, first, count), "neural_get_records")
        return out

    def capture(self, capacity: int, stride: int = 1) -> None:
        self._check(self.fn["neural_capture"](self.r.ctx, self.h, capacity, stride), "neural_capture")

    def stop_capture(self) -> None:
        self._check(self.fn["neural_capture"](self.r.ctx, self.h, 0, 1), "neural_capture")

    def record_count(self) -> int:
        n = C.c_int64(0)
        self._check(self.fn["neural_record_count"](self.h, C.byref(n)), "neural_record_count")
        return n.value

    # -- compute
    def train(self, steps: int, batch: int, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999,
              eps: float = 1e-8, seed: int = 7) -> float:
        tp = _TrainParams(steps, batch, lr, beta1, beta2, eps, seed)
        loss = C.c_float(0)
        self._check(self.fn["neural_train"](self.h, C.byref(tp), C.byref(loss)), "neural_train")
        return float(loss.value)

    def fit(self, steps: int, batch: int, lr: float = 3e-3, chunks: int = 10, seed: int = 7) -> float:
        """`steps` Adam steps with a cosine-decayed learning rate (held constant within each of
        `chunks` equal chunks, floor 2% of `lr`). Returns the last batch loss."""
        loss = float("nan")
        per = max(1, steps // chunks)
        for c in range(chunks):
            f = 0.5 * (1.0 + np.cos(np.pi * c / chunks))
            loss = self.train(per, batch, lr=float(max(lr * f, lr * 0.02)), seed=seed + c)
        return loss

    def gradients(self, first: int, count: int):
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float(0)
        self._check(self.fn["neural_gradients"](self.h, first, count, g.ctypes.data, C.byref(loss)),
                    "neural_gradients")
        return g, float(loss.value)

    def infer(self, first: int = 0, count: Optional[int] = None) -> np.ndarray:
        if count is None:
            count = self.record_count() - first
        out = np.zeros((count, 3), np.float32)
        self._check(self.fn["neural_infer"](self.h, first, count, out.ctypes.data), "neural_infer")
        return out

    def bind(self, program: A.ShaderProgram) -> None:
        self._check(self.fn["program_set_neural_shader"](self.r.ctx, program.handle, self.h),
                    "program_set_neural_shader")

    @staticmethod
    def set_test_flags(renderer: A.Renderer, flags: int) -> None:
        """Test hook: flag 1 makes every completed tensor-core wait of the neural shading kernels
        report a timeout (sticky flag bit 6, Renderer.getOverflow)."""
        st = _bind(renderer.lib.cdll)["neural_set_test_flags"](renderer.ctx, flags)
        if st != 0:
            raise A.SoftGLError(st, "sglc_neural_set_test_flags", "invalid flags")

    @staticmethod
    def unbind(renderer: A.Renderer, program: A.ShaderProgram) -> None:
        fns = _bind(renderer.lib.cdll)
        st = fns["program_set_neural_shader"](renderer.ctx, program.handle, None)
        if st != 0:
            raise A.SoftGLError(st, "sglc_program_set_neural_shader", "unbind failed")


def psnr(a: np.ndarray, b: np.ndarray, peak: float = 255.0) -> float:
    d = a.astype(np.float64) - b.astype(np.float64)
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def set_view(inst: S.SceneInstance, blocks: Dict[str, bytes]) -> None:
    """Point an instance at another view of the same scene: re-upload its uniform blocks (camera,
    light); geometry and textures are shared."""
    _set_blocks(inst, blocks)


def pbr_programs(inst: S.SceneInstance) -> List[A.ShaderProgram]:
    return [prog for objs, p in zip(inst.draws, inst.scene.passes) for (vao, prog, res, ps), d in zip(objs, p.draws)
            if d.shading == A.Shading_PBR]


@dataclass
class NeuralReport:
    records: int
    capture_stride: int
    train_steps: int
    final_loss: float
    psnr_views: List[float] = field(default_factory=list)
    maxabs_views: List[int] = field(default_factory=list)
    psnr_without: List[float] = field(default_factory=list)
    psnr_untrained: List[float] = field(default_factory=list)
    bound: bool = False
    capture_s: float = 0.0
    train_s: float = 0.0

    @property
    def psnr_mean(self) -> float:
        return float(np.mean(self.psnr_views)) if self.psnr_views else float("nan")


def _resolved(inst: S.SceneInstance) -> np.ndarray:
    o = inst.outputs()
    return o.get("resolved", o["color"])


def train_neural_ibl(renderer: A.Renderer, scene_kwargs: Optional[dict] = None, train_views: int = 64,
                     test_views: int = 16, records: int = 1 << 22, steps: int = 6000, batch: int = 1 << 14,
                     lr: float = 3e-3, seed: int = 1, threshold_db: float = 40.0, baselines: bool = True,
                     inst: Optional[S.SceneInstance] = None, net: Optional[NeuralShader] = None):
    """Capture fragments of `train_views` orbit views of the PBR scene rendered by the plain shader,
    train the network, compare on `test_views` held-out views, and bind it to the scene's PBR
    program if the lowest held-out PSNR reaches `threshold_db` (else the plain shader stays bound).
    Returns (instance, network, report)."""
    kw = dict(scene_kwargs or {})
    seed_scene = kw.get("seed", 3000)
    width, height = kw.get("width", 1920), kw.get("height", 1080)
    views = lambda v: S.pbr_view_blocks(seed_scene, v, width, height)
    if inst is None:
        inst = S.SceneInstance(renderer, S.config_pbr(**kw))
    progs = pbr_programs(inst)
    if net is None:
        net = NeuralShader(renderer, seed)
    for prog in progs:
        NeuralShader.unbind(renderer, prog)
    # fragments per view, for the capture stride
    renderer.setStatsLevel(2)
    set_view(inst, views(0))
    inst.render()
    frags = int(renderer.drawStats()["fragments_shaded"])
    renderer.setStatsLevel(0)
    stride = max(1, int(np.ceil(train_views * frags / float(records))))
    t0 = time.perf_counter()
    net.capture(records, stride)
    for v in range(train_views):
        set_view(inst, views(v))
        inst.render()
    renderer.waitIdle()
    net.stop_capture()
    n = net.record_count()
    capture_s = time.perf_counter() - t0
    untrained = net.get_params()
    t0 = time.perf_counter()
    loss = net.fit(steps, batch, lr=lr, seed=seed)
    rep = NeuralReport(n, stride, steps, loss, capture_s=capture_s, train_s=time.perf_counter() - t0)
    test = range(train_views, train_views + test_views)
    for v in test:
        set_view(inst, views(v))
        for prog in progs:
            NeuralShader.unbind(renderer, prog)
        inst.render()
        plain = _resolved(inst)
        for prog in progs:
            net.bind(prog)
        inst.render()
        neural = _resolved(inst)
        rep.psnr_views.append(psnr(neural[..., :3], plain[..., :3]))
        rep.maxabs_views.append(int(np.max(np.abs(neural[..., :3].astype(np.int32) - plain[..., :3]))))
    if baselines:
        trained = net.get_params()
        # the method without the network: the shader's own non-IBL ambient term (u_enableIBL = 0)
        for v in test:
            blocks = views(v)
            for prog in progs:
                NeuralShader.unbind(renderer, prog)
            set_view(inst, blocks)
            inst.render()
            plain = _resolved(inst)
            without = dict(blocks)
            without["UniformsMaterial"] = _without_ibl(blocks["UniformsMaterial"])
            set_view(inst, without)
            inst.render()
            rep.psnr_without.append(psnr(_resolved(inst)[..., :3], plain[..., :3]))
            set_view(inst, blocks)
            net.set_params(untrained)
            for prog in progs:
                net.bind(prog)
            inst.render()
            rep.psnr_untrained.append(psnr(_resolved(inst)[..., :3], plain[..., :3]))
            net.set_params(trained)
    rep.bound = min(rep.psnr_views) >= threshold_db
    set_view(inst, views(0))
    for prog in progs:
        if rep.bound:
            net.bind(prog)
        else:
            NeuralShader.unbind(renderer, prog)
    return inst, net, rep


@dataclass
class MaterialDecision:
    """Whether one material keeps the network: its held-out views, plain against neural."""
    name: str
    psnr_views: List[float]
    maxabs_views: List[int]
    threshold_db: float

    @property
    def psnr_min(self) -> float:
        return float(min(self.psnr_views))

    @property
    def bound(self) -> bool:
        return self.psnr_min >= self.threshold_db


def evaluate_material(renderer: A.Renderer, net: NeuralShader, name: str, scene_kwargs: dict,
                      views: Sequence[int], threshold_db: float = 40.0) -> MaterialDecision:
    """Held-out views of one material (the textures and IBL maps of `S.config_pbr(**scene_kwargs)`,
    e.g. another environment variant) drawn by the plain shader and with the network bound. The
    viewer maps a shader and its resources per material (Viewer.cpp:628, setupMaterial); the network
    is kept for a material only if its lowest PSNR over the views reaches `threshold_db`."""
    kw = dict(scene_kwargs)
    inst = S.SceneInstance(renderer, S.config_pbr(**kw))
    progs = pbr_programs(inst)
    seed = kw.get("seed", 3000)
    w, h = kw.get("width", 1920), kw.get("height", 1080)
    ps, mx = [], []
    for v in views:
        set_view(inst, S.pbr_view_blocks(seed, v, w, h))
        for prog in progs:
            NeuralShader.unbind(renderer, prog)
        inst.render()
        plain = _resolved(inst)
        for prog in progs:
            net.bind(prog)
        inst.render()
        neural = _resolved(inst)
        ps.append(psnr(neural[..., :3], plain[..., :3]))
        mx.append(int(np.max(np.abs(neural[..., :3].astype(np.int32) - plain[..., :3]))))
    for prog in progs:
        NeuralShader.unbind(renderer, prog)
    renderer.waitIdle()
    return MaterialDecision(name, ps, mx, threshold_db)


def bind_per_material(net: NeuralShader, programs_by_material: Dict[str, Sequence[A.ShaderProgram]],
                      decisions: Dict[str, MaterialDecision]) -> Dict[str, bool]:
    """Bind the network to the programs of every material that keeps it; the others keep (or get
    back) the plain shader. Returns material -> network bound."""
    out = {}
    for name, progs in programs_by_material.items():
        keep = decisions[name].bound
        for prog in progs:
            if keep:
                net.bind(prog)
            else:
                NeuralShader.unbind(net.r, prog)
        out[name] = keep
    return out


def _without_ibl(material: bytes) -> bytes:
    b = bytearray(material)
    b[4:8] = (0).to_bytes(4, "little")   # u_enableIBL, the second int of UniformsMaterial (PbrSoft.h:43-45)
    return bytes(b)


def _set_blocks(inst: S.SceneInstance, blocks: Dict[str, bytes]) -> None:
    for objs in inst.draws:
        for vao, prog, res, ps in objs:
            for ub in res.blocks.values():
                if ub.name in blocks:
                    ub.setData(blocks[ub.name])


def main(argv=None) -> None:
    """`python -m softglrender_gb300.neural [--width W --height H --steps N]`: capture, train and
    evaluate the neural IBL shader on a PBR scene, then render it with the network bound."""
    import argparse
    import json
    from . import RendererCUDA
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=480)
    ap.add_argument("--height", type=int, default=270)
    ap.add_argument("--views", type=int, default=8)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--frames", type=int, default=3)
    a = ap.parse_args(argv)
    r = RendererCUDA(0)
    kw = dict(width=a.width, height=a.height, lon=128, lat=64, tex=256, prefilter=128, irradiance=16)
    inst, net, rep = train_neural_ibl(r, kw, train_views=a.views, test_views=2, records=1 << 18, steps=a.steps,
                                      batch=1 << 14)
    for prog in pbr_programs(inst):
        net.bind(prog)
    for _ in range(a.frames):
        inst.render()
    r.waitIdle()
    print(json.dumps({"records": rep.records, "psnr_db": [round(x, 2) for x in rep.psnr_views],
                      "loss": rep.final_loss, "bound": rep.bound}))
    net.destroy()
    r.destroy()


if __name__ == "__main__":
    main()
