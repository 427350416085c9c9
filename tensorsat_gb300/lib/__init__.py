"""Libraries of boxes and diagrams: binary circuits and CNF instances."""
