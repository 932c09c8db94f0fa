"""GB300-native projection/backprojection engine for TomoJ: the Projector surface on CUDA kernels."""
