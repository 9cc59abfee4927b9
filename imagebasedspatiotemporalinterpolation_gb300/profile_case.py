"""Small, fixed workloads for kernel profiles (one launch of each hot kernel).

    python -m imagebasedspatiotemporalinterpolation_gb300.profile_case [--case all|plain|learned|pairs]
                                                                     [--arith reference_gpu|ieee]

plain   one batched call (isti_render_batch, chained) at 1920x1080: main camera plus aux
        cameras at +-0.3 m (6 source views), soft shadows, t = 0.25 / 0.5 / 0.75; one launch
        each of init_kernel, splat_kernel and reproj_kernel, in the arithmetic --arith names
        (default: the reference's GPU arithmetic, as the benchmark line).
learned one learned-initialiser call (isti_render_learned, trained weights, 1 iteration) at
        1920x1080, main camera only, 3 frames: the network's conv kernels, keyframe_kernel,
        learned_kernel and the fallback kernels.
pairs   one isti_render_pairs call over 4 keyframe pairs at 1920x1080 (main camera, 3 frames
        each): one launch of batch_kernel.

Each case runs once after one untimed warm-up call of the same case, so a profiler selects
the second launch of a kernel with `-s 1 -c 1` (learned: the network runs once per call).
Inputs are the seeded procedural scenes of scene.Sequence; about 1 GB is resident.
"""
from __future__ import annotations

import argparse
import sys


def _plain(torch, seq_cls, frame_cls, renderer_cls, arith):
    seq = seq_cls(1920, 1080, 2, seed=2024, aux_offsets=(-0.3, 0.3), shadows=True)
    frame = frame_cls.from_host(seq.frame(0))
    clients = [seq.client(0, b) for b in (1, 2, 3)]
    outs = [torch.zeros((1080, 1920, 4), dtype=torch.uint8, device="cuda") for _ in clients]
    r = renderer_cls()
    r.set_arithmetic(arith)
    for _ in range(2):
        r.render_batch(outs, clients, frame, chain=True)
    torch.cuda.synchronize()
    status = r.device_status()
    r.close()
    return status


def _learned(torch, seq_cls, frame_cls, renderer_cls, arith):
    from . import train_flownet as T
    net = T.load()
    seq = seq_cls(1920, 1080, 2, seed=T.EVAL_SEED_BASE + 7, n_spheres=120, max_speed=1.0, max_rot_deg=5.0, max_step_m=0.1)
    frame = frame_cls.from_host(seq.frame(0))
    clients = [seq.client(0, b) for b in (1, 2, 3)]
    outs = [torch.zeros((1080, 1920, 4), dtype=torch.uint8, device="cuda") for _ in clients]
    r = renderer_cls()
    for _ in range(2):
        r.render_learned(outs, clients, frame, net, 1)
    torch.cuda.synchronize()
    status = r.device_status() | net.device_status()
    r.close()
    net.close()
    return status


def _pairs(torch, seq_cls, frame_cls, renderer_cls, arith):
    seq = seq_cls(1920, 1080, 5, seed=77)
    jobs = []
    for p in range(4):
        frame = frame_cls.from_host(seq.frame(p))
        clients = [seq.client(p, b) for b in (1, 2, 3)]
        outs = [torch.zeros((1080, 1920, 4), dtype=torch.uint8, device="cuda") for _ in clients]
        jobs.append((outs, clients, frame))
    r = renderer_cls()
    for _ in range(2):
        r.render_pairs(jobs)
    torch.cuda.synchronize()
    status = r.device_status()
    r.close()
    return status


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=["all", "plain", "learned", "pairs"], default="all")
    ap.add_argument("--arith", choices=["reference_gpu", "ieee"], default="reference_gpu",
                    help="arithmetic of the plain case (the learned and pairs cases are IEEE)")
    args = ap.parse_args(argv)
    import torch

    from . import native
    arith = native.ARITH_REFERENCE_GPU if args.arith == "reference_gpu" else native.ARITH_IEEE

    from .renderer import DeviceFrame, Renderer
    from .scene import Sequence
    torch.cuda.set_device(0)
    cases = {"plain": _plain, "learned": _learned, "pairs": _pairs}
    names = list(cases) if args.case == "all" else [args.case]
    bad = 0
    for name in names:
        status = cases[name](torch, Sequence, DeviceFrame, Renderer, arith)
        print(f"{name}: device status {status}", flush=True)
        bad |= status
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
