"""Regenerates the golden vectors in tests/golden from the reference's own PyTorch
oracles. Run here, where the reference is mounted (it is not on GPU machines):

    python tests/golden/make_golden.py --reference <the reference checkout>

(or set DIORAMA_REFERENCE to the checkout instead of passing --reference).

1. backward.json and loss.json: reference/backward_reference.py and
   reference/loss_reference.py are imported and their main() re-run (writing to
   a scratch path); the result must equal the reference's committed fixtures
   (src/checks/fixtures/*.json) to 1e-12 before it is copied here.
2. oracle/chunked.py (the tile-chunked float64 renderer) is checked against the
   reference's dense render() on the backward fixture scene and on a 64x48,
   300-Gaussian scene: images and gradients must agree to 1e-10.
3. random_16k.npz: the 16,384-Gaussian random scene (16,384 Gaussians of seed 0, 256x256, SH
   degree 3, black background) against a photo rendered from seed 1 and
   quantized to rgba8: the float64 image, loss_reference.loss, and autograd
   gradients with respect to the activated parameters.
4. fd_20.npz: oracle/chunked.py's float64 loss is checked against
   reference/loss_reference.py's; then central finite differences (step 1e-6)
   of that loss of a 20-Gaussian, SH-degree-3 scene for all 59 trainable values
   per Gaussian, with autograd beside them (the two must agree to 1e-6).
   `--only-fd` runs this step alone.
"""

from __future__ import annotations

import argparse
import importlib.util
import json
import math
import os
import sys
import tempfile
import time
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from diorama_gb300 import scenes  # noqa: E402
from oracle import chunked  # noqa: E402


def load_module(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def regenerate(module, fixture: Path, out: Path) -> float:
    with tempfile.TemporaryDirectory() as tmp:
        module.FIXTURE = Path(tmp) / fixture.name
        module.main()
        fresh = json.loads(module.FIXTURE.read_text())
    committed = json.loads(fixture.read_text())
    worst = 0.0

    def compare(a, b):
        nonlocal worst
        if isinstance(a, dict):
            for k in a:
                if k != "finiteDifferenceError":
                    compare(a[k], b[k])
        elif isinstance(a, list):
            assert len(a) == len(b)
            for x, y in zip(a, b):
                compare(x, y)
        elif isinstance(a, (int, float)) and not isinstance(a, bool):
            worst = max(worst, abs(a - b))

    compare(fresh, committed)
    assert worst < 1e-12, f"{fixture.name} does not reproduce: {worst}"
    out.write_text(json.dumps(fresh))
    return worst


def check_chunked(br) -> None:
    torch.set_default_dtype(torch.float64)
    d = json.loads((HERE / "backward.json").read_text())
    W, H = d["viewport"]
    g = d["gaussians"]
    params = [
        torch.tensor([x["position"] for x in g]), torch.tensor([x["scale"] for x in g]),
        torch.tensor([x["rotation"] for x in g]), torch.tensor([x["opacity"] for x in g]),
        torch.tensor([x["color"] for x in g]), torch.tensor(d["shRest"]).reshape(-1, 15, 3),
    ]
    view, proj = br.as_matrix(d["view"]), br.as_matrix(d["proj"])
    bg = torch.tensor(d["background"])
    cases = [(params, view, proj, bg, W, H)]
    gen = torch.Generator().manual_seed(5)
    n = 300
    rnd = lambda shape, lo, hi: lo + (hi - lo) * torch.rand(shape, generator=gen)  # noqa: E731
    params2 = [rnd((n, 3), -1, 1), rnd((n, 3), 0.03, 0.3), torch.randn((n, 4), generator=gen), rnd((n,), 0.2, 0.95),
               rnd((n, 3), 0.1, 0.9), rnd((n, 15, 3), -0.1, 0.1)]
    view2 = br.as_matrix([float(v) for v in br.look_at([2.0, 1.0, 3.5], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0])])
    proj2 = br.as_matrix(br.perspective(0.9, 64 / 48, 0.1, 100))
    cases.append((params2, view2, proj2, torch.tensor([0.2, 0.1, 0.3]), 64, 48))
    for prm, v, p, b, w, h in cases:
        br.WIDTH, br.HEIGHT, br.SH_DEGREE = w, h, 3
        weights = torch.rand((w * h, 3), generator=gen) - 0.5
        leaves_a = [x.clone().requires_grad_(True) for x in prm]
        ia = br.render(leaves_a, v, p, b)
        (ia * weights).sum().backward()
        leaves_b = [x.clone().requires_grad_(True) for x in prm]
        ib = chunked.render(leaves_b, v, p, b, w, h, 3)
        (ib * weights).sum().backward()
        err = (ia - ib).abs().max().item()
        gerr = max((la.grad - lb.grad).abs().max().item() / max(la.grad.abs().max().item(), 1e-30)
                   for la, lb in zip(leaves_a, leaves_b))
        print(f"chunked vs reference render {w}x{h}: image {err:.2e}, gradients {gerr:.2e} (relative)")
        assert err < 1e-10 and gerr < 1e-10


def make_random_16k(lr) -> None:
    torch.set_default_dtype(torch.float64)
    raw, sh, cam = scenes.random_scene_16k(seed=0)
    raw_t, sh_t = scenes.random_gaussians(16384, seed=1)
    view, proj = chunked.as_matrix(cam.view), chunked.as_matrix(cam.proj)
    W, H = cam.viewport
    bg = torch.zeros(3)

    def leaves(r, s):
        act = scenes.activate64(r).astype(np.float32).astype(np.float64)  # the float32 values the GPU is given
        t = torch.from_numpy
        return [t(act[:, 0:3]), t(act[:, 4:7]), t(act[:, 8:12]), t(act[:, 3]), t(act[:, 12:15]),
                t(s.astype(np.float64).reshape(-1, 15, 3))]

    start = time.time()
    with torch.no_grad():
        photo = chunked.render(leaves(raw_t, sh_t), view, proj, bg, W, H, 3)
    target = np.full((H * W, 4), 255, np.uint8)
    target[:, :3] = np.round(np.clip(photo.numpy(), 0, 1) * 255).astype(np.uint8)
    prm = [x.clone().requires_grad_(True) for x in leaves(raw, sh)]
    image = chunked.render(prm, view, proj, bg, W, H, 3)
    render = image.reshape(H, W, 3).permute(2, 0, 1)
    y = torch.from_numpy(target[:, :3].astype(np.float64) / 255).reshape(H, W, 3).permute(2, 0, 1)
    value = lr.loss(render, y)
    value.backward()
    print(f"random 16k scene: loss {value.item():.10f} in {time.time() - start:.1f} s")
    names = ["position", "scale", "rotation", "opacity", "color", "sh"]
    np.savez_compressed(
        HERE / "random_16k.npz",
        target_rgba8=target.reshape(H, W, 4),
        image=image.detach().numpy().astype(np.float32),
        loss=np.float64(value.item()),
        **{f"grad_{n}": p.grad.numpy().astype(np.float32) for n, p in zip(names, prm)},
    )


FD_VIEWPORT = (40, 32)
FD_GROUPS = [("position", 3), ("scale", 3), ("rotation", 4), ("opacity", 1), ("color", 3), ("sh", 45)]


def check_loss(lr) -> None:
    """oracle/chunked.py's float64 loss against reference/loss_reference.py's."""
    gen = torch.Generator().manual_seed(9)
    for h, w in ((23, 37), (32, 40)):
        target = torch.randint(0, 256, (3, h, w), generator=gen) / 255
        render = (target + 0.2 * torch.randn((3, h, w), generator=gen)).clamp(0, 1)
        err = abs(lr.loss(render, target).item() - chunked.loss(render, target).item())
        print(f"chunked loss vs reference loss {w}x{h}: {err:.1e}")
        assert err < 1e-14


def make_fd_20(br) -> None:
    """fd_20.npz: central finite differences (step 1e-6, float64) of
    loss(render(scene), photo) for every one of the 59 trainable values of 20
    Gaussians with SH degree 3 (position, scale, rotation, opacity, colour: the
    activated layout the renderer is given; the 45 SH coefficients), with
    oracle/chunked.py's renderer and loss. The scene's values are float32 (the
    numbers the GPU is given), evaluated in float64. Autograd gradients are stored
    beside them; the two must agree to 1e-6 of each group's largest (no
    threshold of the blend is crossed within a step)."""
    torch.set_default_dtype(torch.float64)
    W, H = FD_VIEWPORT
    gen = torch.Generator().manual_seed(20)
    uniform = lambda shape, lo, hi: lo + (hi - lo) * torch.rand(shape, generator=gen)  # noqa: E731

    def scene(n):
        prm = [uniform((n, 3), -0.8, 0.8), uniform((n, 3), 0.1, 0.35), torch.randn((n, 4), generator=gen),
               uniform((n,), 0.35, 0.85), uniform((n, 3), 0.45, 0.75), uniform((n, 15, 3), -0.05, 0.05)]
        return [p.to(torch.float32).to(torch.float64) for p in prm]

    params = scene(20)
    truth = scene(24)
    view_list = [float(v) for v in br.look_at([1.2, 0.8, 3.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0])]
    proj_list = br.perspective(math.radians(50), W / H, 0.1, 100)
    view_list = [float(np.float32(v)) for v in view_list]
    proj_list = [float(np.float32(v)) for v in proj_list]
    view, proj = chunked.as_matrix(view_list), chunked.as_matrix(proj_list)
    bg = torch.tensor([0.1, 0.2, 0.3]).to(torch.float32).to(torch.float64)
    with torch.no_grad():
        photo = chunked.render(truth, view, proj, bg, W, H, 3)
    target = np.full((H * W, 4), 255, np.uint8)
    target[:, :3] = np.round(np.clip(photo.numpy(), 0, 1) * 255).astype(np.uint8)
    y = torch.from_numpy(target[:, :3].astype(np.float64) / 255).reshape(H, W, 3).permute(2, 0, 1)

    def loss_of(values):
        image = chunked.render(values, view, proj, bg, W, H, 3)
        return chunked.loss(image.reshape(H, W, 3).permute(2, 0, 1), y)

    leaves = [p.clone().requires_grad_(True) for p in params]
    value = loss_of(leaves)
    value.backward()
    start = time.time()
    step = 1e-6
    fd = []
    with torch.no_grad():
        for index, p in enumerate(params):
            flat = p.flatten()
            estimate = torch.zeros_like(flat)
            for k in range(flat.numel()):
                nudged = list(params)
                up = flat.clone()
                up[k] += step
                nudged[index] = up.reshape(p.shape)
                hi = loss_of(nudged)
                down = flat.clone()
                down[k] -= step
                nudged[index] = down.reshape(p.shape)
                lo = loss_of(nudged)
                estimate[k] = (hi - lo) / (2 * step)
            fd.append(estimate.reshape(p.shape))
    names = ["position", "scale", "rotation", "opacity", "color", "sh"]
    disagreement = {}
    for name, f, leaf in zip(names, fd, leaves):
        disagreement[name] = ((f - leaf.grad).abs().max() / leaf.grad.abs().max()).item()
    print(f"fd_20: loss {value.item():.10f}, {time.time() - start:.0f} s of finite differences; autograd "
          f"disagrees by {max(disagreement.values()):.1e} of a group's largest ({disagreement})")
    assert max(disagreement.values()) < 1e-6
    n = params[0].shape[0]
    gaussians = np.zeros((n, 16), np.float32)
    gaussians[:, 0:3] = params[0].numpy()
    gaussians[:, 4:7] = params[1].numpy()
    gaussians[:, 8:12] = params[2].numpy()
    gaussians[:, 3] = params[3].numpy()
    gaussians[:, 12:15] = params[4].numpy()
    np.savez_compressed(
        HERE / "fd_20.npz", gaussians=gaussians, sh=params[5].numpy().astype(np.float32).reshape(n, 45),
        view=np.array(view_list), proj=np.array(proj_list), viewport=np.array([W, H]), background=bg.numpy(),
        target_rgba8=target, loss=np.float64(value.item()),
        **{f"fd_{k}": f.numpy() for k, f in zip(names, fd)},
        **{f"autograd_{k}": leaf.grad.numpy() for k, leaf in zip(names, leaves)})


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("DIORAMA_REFERENCE"),
                    help="the reference project's checkout (default: $DIORAMA_REFERENCE)")
    ap.add_argument("--skip-random-16k", action="store_true")
    ap.add_argument("--only-fd", action="store_true", help="only check the loss and remake fd_20.npz")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give the reference checkout with --reference or DIORAMA_REFERENCE")
    ref = Path(args.reference)
    fixtures = ref / "src" / "checks" / "fixtures"
    br = load_module(ref / "reference" / "backward_reference.py", "backward_reference")
    if args.only_fd:
        check_loss(load_module(ref / "reference" / "loss_reference.py", "loss_reference"))
        make_fd_20(br)
        return
    w = regenerate(br, fixtures / "backward.json", HERE / "backward.json")
    print(f"backward.json reproduces the reference fixture to {w:.1e}")
    lr = load_module(ref / "reference" / "loss_reference.py", "loss_reference")
    w = regenerate(lr, fixtures / "loss.json", HERE / "loss.json")
    print(f"loss.json reproduces the reference fixture to {w:.1e}")
    check_chunked(br)
    check_loss(lr)
    make_fd_20(br)
    if not args.skip_random_16k:
        make_random_16k(lr)


if __name__ == "__main__":
    main()
