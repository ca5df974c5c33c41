"""Host-side logic of the proposal network: layer-list validation and the
layer list stored with the weights (no kernels run)."""

import numpy as np
import pytest

from leopard_em_gb300 import proposal as pr

WIDE = [("conv", 12, 48, 2, True), ("conv", 48, 96, 2, True), ("conv", 96, 128, 2, True),
        ("conv", 128, 128, 2, True), ("conv", 128, 128, 1, True), ("fc", 2048, 1152, 1, True),
        ("fc", 1152, 256, 1, True), ("fc", 256, 7, 1, False)]
NARROW = [("conv", 12, 32, 2, True), ("conv", 32, 64, 2, True), ("conv", 64, 96, 2, True),
          ("conv", 96, 128, 2, True), ("conv", 128, 128, 1, True), ("fc", 2048, 512, 1, True),
          ("fc", 512, 128, 1, True), ("fc", 128, 7, 1, False)]


def test_default_network_shape():
    net = pr.ProposalNet("cpu")
    assert net.layers == [tuple(l) for l in pr.LAYERS] == WIDE and net.n_params == 3110103
    assert net.n_params == sum(w.numel() + b.numel() for w, b in zip(net.w, net.b))


@pytest.mark.parametrize("bad", [
    [("conv", 11, 32, 2, True)] + WIDE[1:],                     # input channels
    WIDE[:1] + [("conv", 48, 160, 2, True)] + WIDE[2:],        # > 128 channels
    WIDE[:5] + [("fc", 2000, 1152, 1, True)] + WIDE[6:],       # flattened size
    WIDE[:7] + [("fc", 256, 6, 1, False)],                     # output width
    WIDE[:2] + [("pool", 96, 96, 2, True)] + WIDE[3:],         # unknown kind
])
def test_bad_layer_lists_are_rejected(bad):
    with pytest.raises(ValueError):
        pr.ProposalNet("cpu", layers=bad)


def test_layer_list_travels_with_the_weights(tmp_path):
    net = pr.ProposalNet("cpu", seed=4, layers=NARROW)
    path = str(tmp_path / "w.npz")
    pr.save_weights(net, path)
    assert pr.stored_layers(path) == NARROW
    back = pr.load_net(path, "cpu")
    assert back.layers == NARROW and back.n_params == net.n_params == 1451335
    for a, b in zip(net.w, back.w):  # stored as float16
        assert np.allclose(a.numpy(), b.numpy(), rtol=1e-3, atol=1e-4)
    with pytest.raises(ValueError):
        pr.load_weights(pr.ProposalNet("cpu"), path)  # shapes of another layer list
