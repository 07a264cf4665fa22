"""Mirror of spinifel.extern: the NUFFT operator class."""
