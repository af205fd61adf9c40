"""Timing and golden-output runs of LibreTT's own CUDA build (test infrastructure)."""
