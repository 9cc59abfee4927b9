"""Trains the learned flow initialiser on the GPU (checkpoint recipe).

Training data are produced on the device, per sample:
  1. a seeded procedural scene (ground plane + U[16, 256] spheres, radius U[0.2, 1.5] m,
     |v| <= 1 m/s) and a keyframe pair 1/30 s apart seen from a camera that rotates by
     up to 5 degrees and moves by up to 10 cm in that interval;
  2. both keyframes ray-cast by isti_scene_raycast (NDC z and object motion);
  3. the plain method (isti_render, mode 0) for a client camera at t in {0.25, 0.5,
     0.75} on the interpolated pose, and from its keys and flows the labels: per
     quarter-resolution pixel the converged source offset in each keyframe
     (isti_learned_labels, NaN where the plain search did not converge);
  4. the network input of the learned path (isti_learned_input).
Each step runs the forward pass, the loss and all gradients on the tcgen05 kernels
(isti_flownet_backward) and one Adam step (isti_flownet_adam).

    python -m imagebasedspatiotemporalinterpolation_gb300.train_flownet --pairs 20000 \\
        --out imagebasedspatiotemporalinterpolation_gb300/weights/flownet.npz

Held-out evaluation seeds start at EVAL_SEED_BASE; training seeds stay below it.
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
import os
import time

import numpy as np

from . import native
from .flownet import FlowNet
from .native import check
from .renderer import DeviceFrame, DeviceView, Renderer, render_info
from .scene import Client, Pose, perspective, view_matrix

EVAL_SEED_BASE = 1 << 30
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "flownet.npz")
KEYFRAME_DT = 1.0 / 30.0
T_VALUES = (0.25, 0.5, 0.75)


def _torch():
    import torch
    return torch


def _cm(m: np.ndarray):
    return (C.c_double * 16)(*np.asarray(m, np.float64).T.reshape(-1).tolist())


class PairSampler:
    """Seeded random scenes and camera pairs (configuration of the learned initialiser's
    training set), ray-cast on the GPU at width x height."""

    def __init__(self, width: int, height: int, max_rot_deg: float = 5.0, max_step_m: float = 0.10,
                 spheres: tuple[int, int] = (16, 256), max_speed: float = 1.0):
        torch = _torch()
        self.width, self.height = width, height
        self.max_rot, self.max_step, self.spheres, self.max_speed = max_rot_deg, max_step_m, spheres, max_speed
        self.proj = perspective(90.0, width / height, 0.1, 100.0)
        self.color = torch.zeros((height, width, 4), dtype=torch.uint8, device="cuda")  # colour is not needed for labels
        self._lib = native.load()

    def sample(self, seed: int):
        """(DeviceFrame, Client) of one training sample."""
        torch = _torch()
        rng = np.random.default_rng(seed)
        n = int(rng.integers(self.spheres[0], self.spheres[1] + 1))
        r = rng.uniform(0.2, 1.5, n)
        c = rng.uniform(-10.0, 10.0, (n, 2))
        sp = rng.uniform(0.0, self.max_speed, n)
        ang = rng.uniform(0.0, 2 * math.pi, n)
        arr = np.stack([c[:, 0], c[:, 1], r, sp * np.cos(ang), sp * np.sin(ang)], 1).astype(np.float32)
        spheres = torch.from_numpy(arr).cuda()
        eye = np.array([rng.uniform(-12, 12), rng.uniform(1.2, 4.0), rng.uniform(-16, -8)])
        pose_a = Pose(eye, rng.uniform(-0.6, 0.6), math.radians(rng.uniform(-20.0, 0.0)))
        d = rng.standard_normal(3)
        d = d / max(1e-9, np.linalg.norm(d)) * rng.uniform(0.0, self.max_step)
        rot = math.radians(rng.uniform(0.0, self.max_rot))
        phi = rng.uniform(0, 2 * math.pi)
        pose_b = Pose(pose_a.eye + d, pose_a.yaw + rot * math.cos(phi), pose_a.pitch + 0.5 * rot * math.sin(phi))
        views = []
        for k, (pose, sign) in enumerate(((pose_a, 1.0), (pose_b, -1.0))):
            vp = self.proj @ view_matrix(pose.eye, pose.yaw, pose.pitch)
            ivp = np.linalg.inv(vp)
            z = torch.empty((self.height, self.width), dtype=torch.float32, device="cuda")
            m = torch.empty((self.height, self.width, 3), dtype=torch.float16, device="cuda")
            check(self._lib.isti_scene_raycast(C.c_void_p(spheres.data_ptr()), n, self.width, self.height, _cm(vp), _cm(ivp),
                                                k * KEYFRAME_DT, sign * KEYFRAME_DT, C.c_void_p(z.data_ptr()), C.c_void_p(m.data_ptr()),
                                                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            views.append(DeviceView(self.color, z, m, viewproj=vp.astype(np.float32), inv_viewproj=ivp.astype(np.float32)))
        t = float(T_VALUES[int(rng.integers(0, len(T_VALUES)))])
        pose_c = pose_a.lerp(pose_b, t)
        vpc = self.proj @ view_matrix(pose_c.eye, pose_c.yaw, pose_c.pitch)
        client = Client(self.width, self.height, float(np.float32(t)), vpc.astype(np.float32),
                        np.linalg.inv(vpc).astype(np.float32))
        return DeviceFrame(views[0], views[1]), client, spheres


def grid(width: int, height: int) -> tuple[int, int]:
    gw, gh = C.c_int32(), C.c_int32()
    check(native.load().isti_learned_grid(width, height, C.byref(gw), C.byref(gh)))
    return gh.value, gw.value


class Batcher:
    """Builds batches of network inputs and plain-method labels on the GPU."""

    def __init__(self, width: int, height: int, batch: int):
        torch = _torch()
        self.sampler = PairSampler(width, height)
        self.hq, self.wq = grid(width, height)
        self.batch = batch
        self.x = torch.empty((batch, self.hq, self.wq, 16), dtype=torch.bfloat16, device="cuda")
        self.label = torch.empty((batch, self.hq, self.wq, 4), dtype=torch.float32, device="cuda")
        self.out = torch.zeros((height, width, 4), dtype=torch.uint8, device="cuda")
        self.renderer = Renderer()
        self._lib = native.load()

    def fill(self, seeds) -> None:
        torch = _torch()
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for i, seed in enumerate(seeds):
            frame, client, _spheres = self.sampler.sample(int(seed))
            self.renderer.render(self.out, client, frame)
            check(self._lib.isti_learned_labels(self.renderer._h, 0, C.c_void_p(self.label[i].data_ptr()), s))
            ri = render_info(client)
            check(self._lib.isti_learned_input(self.renderer._h, 1, C.byref(ri), C.byref(frame.to_c()),
                                               C.c_void_p(self.x[i].data_ptr()), s))


def train(pairs: int, batch: int = 4, width: int = 1920, height: int = 1080, lr: float = 1e-3, seed: int = 0, log_every: int = 100,
          net: FlowNet | None = None, time_limit_s: float | None = None, verbose: bool = True) -> tuple[FlowNet, list]:
    """Trains on `pairs` seeded samples (one t per keyframe pair); cosine learning-rate decay."""
    torch = _torch()
    net = net or FlowNet(seed=seed)
    b = Batcher(width, height, batch)
    steps = max(1, pairs // batch)
    hist = []
    t0 = time.time()
    for step in range(steps):
        seeds = [seed * 1_000_003 + step * batch + i for i in range(batch)]
        b.fill(seeds)
        net.backward(b.x, b.label)
        cur = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        net.adam(cur)
        if (step + 1) % log_every == 0 or step == steps - 1:
            loss = net.loss()
            hist.append((step + 1, loss, time.time() - t0))
            if verbose:
                print(f"step {step + 1}/{steps} loss {loss:.5f} lr {cur:.2e} {time.time() - t0:.1f}s", flush=True)
        if time_limit_s is not None and time.time() - t0 > time_limit_s:
            break
    torch.cuda.synchronize()
    if net.device_status() != 0:
        raise RuntimeError("a bounded wait in a network kernel gave up during training")
    return net, hist


def save(net: FlowNet, path: str, meta: dict | None = None) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, params=net.params().cpu().numpy(), **{k: np.array(v) for k, v in (meta or {}).items()})


def load(path: str = DEFAULT_WEIGHTS, seed: int = 0) -> FlowNet:
    torch = _torch()
    data = np.load(path)
    net = FlowNet(seed=seed)
    net.set_params(torch.from_numpy(data["params"]))
    return net


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--time-limit", type=float, default=None, help="stop after this many seconds (the schedule keeps --pairs)")
    args = ap.parse_args()
    net, hist = train(args.pairs, args.batch, args.width, args.height, args.lr, args.seed, time_limit_s=args.time_limit)
    save(net, args.out, {"pairs": args.pairs, "batch": args.batch, "width": args.width, "height": args.height, "lr": args.lr,
                         "seed": args.seed, "steps_run": hist[-1][0] if hist else 0, "loss_history": np.array(hist)})
    print(f"saved {args.out}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
