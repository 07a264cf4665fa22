"""Run parameters for the hot path, with the reference's setting names.

The reference reads a TOML file through the SpinifelSettings singleton
(spinifel/settings.py:167-848).  Only the fields the slicing / matching /
merge / phasing path reads are mirrored here, as a plain dataclass with the same names
and derived values:
  Mquat = 20 * oversampling, M = 4 Mquat + 1, M_ups = 2 M
(spinifel/settings.py:805-826) and
  reduced_det_shape = det_shape with the last two axes divided by
  2**(N_clipping + N_binning) (spinifel/settings.py:834-838).
M and M_ups can be overridden for the synthetic workloads (41^3, 151^3).
"""
from __future__ import annotations

from dataclasses import dataclass, field


@dataclass
class Settings:
    N_orientations: int = 1000
    N_batch_size: int = 1000
    det_shape: tuple = (4, 512, 512)
    N_clipping: int = 1
    N_binning: int = 4
    oversampling: int = 1
    N_images_per_rank: int = 10
    use_single_prec: bool = True
    use_cuda: bool = True
    solve_ac_maxiter: int = 100
    verbose: bool = False
    M_override: int | None = None
    M_ups_override: int | None = None
    Mquat_override: int | None = None
    # phase retrieval (spinifel/settings.py:388-412)
    beta: float = 0.9
    cutoff: float = 5e-2
    nER: int = 10
    nHIO: int = 5
    N_phase_loops: int = 5
    reduced_det_shape_override: tuple | None = field(default=None)

    @property
    def Mquat(self) -> int:
        return self.Mquat_override if self.Mquat_override else int(self.oversampling * 20)

    @property
    def M(self) -> int:
        return self.M_override if self.M_override else 4 * self.Mquat + 1

    @property
    def M_ups(self) -> int:
        return self.M_ups_override if self.M_ups_override else 2 * self.M

    @property
    def N_binning_tot(self) -> int:
        return self.N_clipping + self.N_binning

    @property
    def reduced_det_shape(self) -> tuple:
        if self.reduced_det_shape_override is not None:
            return tuple(self.reduced_det_shape_override)
        d = tuple(self.det_shape)
        return d[:-2] + (d[-2] // 2 ** self.N_binning_tot, d[-1] // 2 ** self.N_binning_tot)


settings = Settings()


def SpinifelSettings() -> Settings:
    """Module-level settings object, mirroring the reference singleton."""
    return settings
