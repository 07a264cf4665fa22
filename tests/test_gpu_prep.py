"""Frame clipping + binning on the GPU (spf_bin_frames_u16) against the
reference's spinifel/prep.py functions run on the same counts (golden):
exact, the sums are integers."""
import os

import numpy as np
import pytest
import torch

from tests.golden import cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_bin_frames_matches_reference(lib):
    from spinifel_gb300.prep import bin_frames

    c = cases.PREP
    g = np.load(os.path.join(GOLD, "golden_prep.npz"))
    f4, f1, _, _ = cases.prep_inputs()
    dev = torch.device("cuda", 0)

    def dev16(a):
        return torch.as_tensor(a.astype(np.int16), device=dev)

    nc, nb = c["n_clip"], c["n_bin"]
    np.testing.assert_array_equal(bin_frames(dev16(f4), nc, nb).cpu().numpy(), g["sum4"])
    np.testing.assert_array_equal(bin_frames(dev16(f4), nc, nb, mean=True).cpu().numpy(),
                                  g["mean4"])
    np.testing.assert_array_equal(bin_frames(dev16(f1), nc, nb).cpu().numpy(), g["sum1"])
    np.testing.assert_array_equal(bin_frames(dev16(f4), 0, nb).cpu().numpy(), g["sum4_noclip"])


def test_bin_frames_full_counts_and_rejections(lib):
    """Counts up to 65535 (uint16 carried as int16 bits) sum exactly; shapes
    that the reference cannot clip or bin are rejected on the host."""
    from spinifel_gb300 import _lib
    from spinifel_gb300.prep import bin2nx2n_sum, bin_frames, clipping

    rng = np.random.default_rng(5)
    raw = rng.integers(0, 65536, (2, 4, 64, 64)).astype(np.uint16)
    got = bin_frames(torch.as_tensor(raw.view(np.int16), device="cuda"), 1, 3).cpu().numpy()
    ref = bin2nx2n_sum(clipping(raw.astype(np.float64), 1), 3)
    np.testing.assert_array_equal(got, ref.astype(np.float32))
    with pytest.raises(_lib.SpfError):
        bin_frames(torch.zeros(1, 2, 16, 16, dtype=torch.int16, device="cuda"), 1, 1)  # 2 panels
    with pytest.raises(_lib.SpfError):
        bin_frames(torch.zeros(1, 4, 12, 12, dtype=torch.int16, device="cuda"), 0, 3)  # 12 % 8
