"""Mirror of spinifel.sequential: the orientation-matching and merge objects
with the reference's call surface, running on libspinifel_gb300."""
