"""Learned plan selection: dataset collection, GPU training, evaluation.

The engine ranks its candidate plans with a small MLP (features of a
candidate -> predicted log time).  This package measures every candidate of
many random problems on the device (the training data), trains the MLP with
the library's own CUDA kernels (librett_c_mlp_*), writes the weight file the
library loads at plan time (librett_gb300/models/plan_mlp.bin), and
evaluates the regret of the choice against the measured best.
"""
