"""Stand-alone sort, mirroring MetalKernelsRadixSort (Astro/RadixSort.swift:24-186).

``RadixSort(max_length).sort(input, input_indices, output, output_indices,
estimated_length, actual_count)`` sorts (uint64 key, uint32 index) pairs
stably, like the reference's ``sort(commandBuffer:input:inputIndices:output:
outputIndices:estimatedLength:actualCountBuffer:)``. Buffers are CUDA tensors
(torch is used only to hold device memory and pass its pointers); the
temporary buffers belong to the sorter, as the reference's tempKeys /
tempIndices do (RadixSort.swift:57-66).
"""
from __future__ import annotations

from ctypes import byref, c_size_t

from ._native import check, lib, ptr


class RadixSort:
    def __init__(self, max_length: int, key_bits: int = 64, device=None):
        import torch

        self.max_length = max_length
        self.key_bits = key_bits
        nbytes = c_size_t()
        check(lib().astro_radix_sort_temp_bytes(max_length, key_bits, byref(nbytes)))
        self.temp = torch.empty(nbytes.value, dtype=torch.uint8, device=device or "cuda")

    def sort(self, input, input_indices, output, output_indices, estimated_length: int,
             actual_count=None, stream: int = 0) -> None:
        """Sort the first count pairs; count is read on the device from
        actual_count (a one-element uint32 CUDA tensor) when given."""
        if estimated_length > self.max_length:
            raise ValueError("estimated_length exceeds the sorter's max_length")
        check(lib().astro_radix_sort(ptr(input), ptr(input_indices), ptr(output),
                                     ptr(output_indices), estimated_length, ptr(actual_count),
                                     self.key_bits, ptr(self.temp), self.temp.numel(), stream))

    def status(self, stream: int = 0) -> None:
        """Wait for `stream` and raise AstroError(ASTRO_ERR_DEVICE_TIMEOUT) if
        the last sort on this sorter's temporaries had a look-back wait give
        up (the NULL stream's sort already reported it from sort())."""
        check(lib().astro_radix_sort_status(ptr(self.temp), stream))
