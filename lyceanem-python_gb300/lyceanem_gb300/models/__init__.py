"""Model-level API with the call shape of lyceanem.models."""
