"""The one-launch Adam against torch.optim.Adam (same update rule)."""
import pytest
import torch

from pointrix_gb300.optim import Adam

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("capturable", [False, True])
def test_adam_matches_torch_over_steps(capturable):
    """Five steps; on steps 2 and 3 a different parameter has no gradient
    (the same number of parameters takes part in both), which must leave that
    parameter and its step count untouched in either mode."""
    g = torch.Generator().manual_seed(0)
    shapes = [(1000, 3), (1000, 16, 3), (1001,), (4,), (3, 4)]
    lrs = [1.6e-4, 2.5e-3, 5e-2, 1e-3, 1e-4]
    a = [torch.randn(s, generator=g).cuda().requires_grad_(True) for s in shapes]
    b = [t.detach().clone().requires_grad_(True) for t in a]
    mine = Adam([{"params": [t], "lr": lr} for t, lr in zip(a, lrs)], eps=1e-15,
                capturable=capturable)
    ref = torch.optim.Adam([{"params": [t], "lr": lr} for t, lr in zip(b, lrs)], eps=1e-15)
    start = [t.detach().clone() for t in b]
    for step in range(5):
        grads = [torch.randn(s, generator=g).cuda() for s in shapes]
        for t, gr in zip(a, grads):
            t.grad = gr.clone()
        for t, gr in zip(b, grads):
            t.grad = gr.clone()
        if step in (2, 3):
            skip = 1 if step == 2 else 2   # a parameter without a gradient is skipped
            a[skip].grad = None
            b[skip].grad = None
        mine.step()
        ref.step()
        # the accumulated update agrees to float32 rounding of the update rule
        for x, y, x0 in zip(a, b, start):
            rel = float((x - y).norm() / (y - x0).norm())
            assert rel < 1e-4, (step, rel)
