"""The fitting loop's checkpoint format (fitting.save_checkpoint /
load_checkpoint) round-trips on the CPU: grids, both Adam moments, the step
count and the extra entries."""
import torch

from binarymeshfitting_gb300.fitting import load_checkpoint, save_checkpoint


def test_checkpoint_roundtrip(tmp_path):
    g = torch.Generator().manual_seed(5)
    dens = torch.randn(3 * 17 ** 3, generator=g)
    state = {"m": torch.randn(dens.shape, generator=g), "v": torch.rand(dens.shape, generator=g),
             "step": torch.tensor([7], dtype=torch.int32)}
    path = str(tmp_path / "ck.pt")
    save_checkpoint(path, dens, state, step=7, lr=0.01)
    d2, s2, extra = load_checkpoint(path, "cpu")
    assert torch.equal(d2, dens) and extra == {"step": 7, "lr": 0.01}
    for k in ("m", "v", "step"):
        assert torch.equal(s2[k], state[k]) and s2[k].dtype == state[k].dtype
