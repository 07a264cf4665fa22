"""A whole SNM generation recorded as one CUDA graph (model set-up, each
orientation batch's slicing, std rescale, distances and running argmin) and
replayed for new models gives the eager indices bit for bit, on the fast FP32
path and at the reference's FP64 precision."""
import numpy as np
import pytest
import torch

from tests.golden import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("single", [True, False])
def test_snm_generation_graph_replay_equals_eager(lib, single):
    from spinifel_gb300 import Settings, synth
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.orientation_matching import SNM

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    s = cases.SNM
    st = Settings(N_orientations=s["n_orient"], N_batch_size=s["batch"],
                  det_shape=s["det_shape"], N_clipping=0, N_binning=0,
                  use_single_prec=single)
    nufft = NUFFT(st, ppr, pdr, ref_orientations=quats)
    snm = SNM(st, slices_, ppr, pdr, nufft)
    ac2 = synth.intensity_model(s["M"], seed=99)
    eager = [snm.match_indices(a).clone() for a in (ac, ac2)]
    snm.capture(ac)
    for _ in range(2):  # each model twice, alternating
        for a, e in zip((ac, ac2), eager):
            assert torch.equal(snm.match_indices_graphed(a), e)
    assert not torch.equal(eager[0], eager[1])  # the two models give different answers
