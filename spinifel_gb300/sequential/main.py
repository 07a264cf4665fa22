"""The sequential M-TIP loop with the reference's structure
(spinifel/sequential/main.py:12-70): merge with random orientations, phase,
then per generation: orientation matching against the phased model, merge
with the matched orientations, phase again.  Every stage runs on the GPU
(slicing + matching, the merge's NUFFTs and CG, phasing); the data come in as
arrays (the reference loads them from HDF5 or psana, absent here)."""
from __future__ import annotations

import time

import numpy as np

from ..extern.nufft_ext import NUFFT
from .autocorrelation import Merge
from .orientation_matching import SNM
from .phasing import phase


def main(settings, pixel_position_reciprocal, pixel_distance_reciprocal, slices_,
         n_generations: int = 10, ref_orientations=None, seed=None, log=None):
    """Returns (ac_phased, support_, rho_, orientations, timings) after
    n_generations (generation 0 included), as the reference's loop leaves them."""
    log = log or (lambda *_: None)
    rng = np.random.default_rng(seed)
    timings = []
    t = time.perf_counter()
    nufft = NUFFT(settings, pixel_position_reciprocal, pixel_distance_reciprocal,
                  ref_orientations=ref_orientations)
    mg = Merge(settings, slices_, pixel_position_reciprocal, pixel_distance_reciprocal, nufft,
               seed=seed)
    snm = SNM(settings, slices_, pixel_position_reciprocal, pixel_distance_reciprocal, nufft)
    ac = mg.solve_ac(0)
    t1 = time.perf_counter()
    ac_phased, support_, rho_ = phase(0, ac, settings=settings, rng=rng)
    t2 = time.perf_counter()
    timings.append({"generation": 0, "merge_s": t1 - t, "phase_s": t2 - t1})
    log(f"generation 0: merge {t1 - t:.2f}s, phase {t2 - t1:.2f}s")
    orientations = None
    for generation in range(1, n_generations):
        t0 = time.perf_counter()
        orientations = snm.slicing_and_match(ac_phased)
        t1 = time.perf_counter()
        ac = mg.solve_ac(generation, orientations, ac_phased)
        t2 = time.perf_counter()
        ac_phased, support_, rho_ = phase(generation, ac, support_, rho_, settings=settings,
                                          rng=rng)
        t3 = time.perf_counter()
        timings.append({"generation": generation, "match_s": t1 - t0, "merge_s": t2 - t1,
                        "phase_s": t3 - t2})
        log(f"generation {generation}: match {t1 - t0:.2f}s, merge {t2 - t1:.2f}s, "
            f"phase {t3 - t2:.2f}s")
    return ac_phased, support_, rho_, orientations, timings
