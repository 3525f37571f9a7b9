"""GB300-native (sm_103a) implementation of the MLegS spectral hot path."""
from .params import MlgParams, make_params, dims_of  # noqa: F401
