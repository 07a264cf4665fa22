"""Single-GPU counterparts of the reference's MPI modules (spinifel/mpi)."""
