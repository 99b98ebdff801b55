"""Convolutional surrogate of exact openness (see openness_cnn)."""
from .openness_cnn import OpennessSurrogate, surrogate_features  # noqa: F401
