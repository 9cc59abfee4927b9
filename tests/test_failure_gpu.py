"""Failure detection on the GPU without a fault: a bounded wait that runs out.

The reprojection kernel stages its splat-key tiles by TMA and waits for them on an
mbarrier with an iteration limit.  The test hook isti_renderer_test_withhold_tile
makes one block announce its tile bytes but issue no copy, so nothing ever
completes its barrier: its wait must give up after the (short) limit, set
ISTI_ERR_TIMEOUT in the device status word and leave without reading a tile or
writing a pixel, while every other block renders as before.  No copy is in
flight for that block, so it leaves nothing behind; the context stays usable and
the next render, with the hook off, is correct again.
"""
import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300 import native
from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence

pytestmark = pytest.mark.gpu

WAIT_LIMIT = 1 << 12  # polls of the barrier before giving up (twice): well under a second


def rule_block_rows(n_views, n_frames=1):
    """Output rows per reprojection block under the fixed launch rule (row pairs = views / (2 frames), 1..3)."""
    return 2 * max(1, min(3, n_views // (2 * n_frames)))


@pytest.mark.parametrize("aux", [(), (-0.3, 0.3)], ids=["main", "aux"])
def test_withheld_tile_times_out_and_only_its_block_is_skipped(cuda, aux):
    import torch
    seq = Sequence(640, 360, 2, seed=905, aux_offsets=aux, shadows=bool(aux))
    frame = DeviceFrame.from_host(seq.frame(0))
    client = seq.client(0, 2)
    prev = torch.full((360, 640, 4), 7, dtype=torch.uint8, device="cuda")
    r = Renderer()
    want = prev.clone()
    r.render(want, client, frame)
    assert r.device_status() == native.ISTI_OK

    # withhold a block whose pixels the normal render writes (main-camera-only renders
    # leave holes, kept from the previous frame)
    rows = rule_block_rows(len(frame.views()))
    written = (want != prev).any(-1)
    blocks = written[: 360 // rows * rows].reshape(360 // rows, rows, 640 // 32, 32).any(3).any(1)
    by, bx = [int(v) for v in torch.nonzero(blocks)[len(torch.nonzero(blocks)) // 2]]
    px, py = bx * 32 + 5, by * rows + rows - 1
    r.test_withhold_tile(px, py, WAIT_LIMIT)
    got = prev.clone()
    r.render(got, client, frame)
    assert r.device_status() == native.ISTI_ERR_TIMEOUT

    x0, y0 = px // 32 * 32, py // rows * rows
    mask = torch.zeros((360, 640), dtype=torch.bool, device="cuda")
    mask[y0:y0 + rows, x0:x0 + 32] = True
    assert torch.equal(got[~mask], want[~mask]), "blocks other than the withheld one changed"
    assert torch.equal(got[mask], prev[mask]), "the withheld block wrote pixels"
    assert bool((want[mask] != prev[mask]).any()), "the block's pixels should normally be rendered"

    r.test_withhold_tile(-1, -1, 0)
    again = prev.clone()
    r.render(again, client, frame)
    assert r.device_status() == native.ISTI_OK
    assert torch.equal(again, want)
    r.close()
