"""Box classes (languages) of tensorsat_gb300: :mod:`.cuda_rel`."""
