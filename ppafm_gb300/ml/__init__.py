"""Machine-learning data generation on the GPU path (ppafm/ml)."""
