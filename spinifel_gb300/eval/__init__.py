"""Reconstruction-quality tools with the reference's surface (eval/fsc.py,
eval/align.py): Fourier shell correlation and volume alignment, the scoring
of candidate rotations and the shell sums on the GPU."""
