"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the vkrt CUDA backend (see oracle.h)."""
