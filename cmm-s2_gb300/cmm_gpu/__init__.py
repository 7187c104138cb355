"""GB300-native CMM hot path: Python side of libcmmgpu.so."""
