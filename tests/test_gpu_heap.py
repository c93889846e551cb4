"""Allocator churn on the GPU: every thread loops malloc, fill, verify, free.

Pass criterion (the allocation part of the point-to-point workload): every
pattern survives until its free, no allocation fails while the heap has room,
every pointer is 16-byte aligned.  Known answers after the allocator tests of
gpu_libs/gpu_malloc/dynamic_allocator/tests.cu:12-120 (sizes, alignment,
round trips).
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("blocks,threads,iters,live,heap_gib", [(1, 32, 50, 4, 1), (152, 256, 64, 8, 8),
                                                               (608, 1024, 32, 8, 16)])
def test_slab_churn_patterns_survive(gpu_built, blocks, threads, iters, live, heap_gib):
    lib = gpu_built.load_library()
    st = gpu_built.malloc_churn(lib, blocks, threads, iters, live=live, seed=blocks * 31 + live,
                                heap_bytes=heap_gib << 30)
    n = blocks * threads * iters
    assert st["allocs"] == n
    assert st["failed"] == 0
    assert st["frees"] == n
    assert st["corrupt"] == 0
    assert st["misaligned"] == 0
    assert 0 < st["malloc_cycles_p50"] <= st["malloc_cycles_p99"]


def test_slab_churn_heap_exhaustion_reports_failures(gpu_built):
    """A heap too small for the live set returns NULL instead of overlapping objects."""
    lib = gpu_built.load_library()
    st = gpu_built.malloc_churn(lib, 152, 256, 16, live=16, seed=5, heap_bytes=64 << 20)
    assert st["failed"] > 0
    assert st["corrupt"] == 0
    assert st["frees"] == st["allocs"] - st["failed"]


def test_cuda_heap_churn_for_comparison(gpu_built):
    """The same loop on CUDA's device malloc (the reference's allocator) stays correct."""
    lib = gpu_built.load_library()
    st = gpu_built.malloc_churn(lib, 38, 256, 8, live=4, seed=9, heap_bytes=1 << 30, cuda_heap=True)
    assert st["corrupt"] == 0
    assert st["frees"] == st["allocs"] - st["failed"]


@pytest.mark.parametrize("nbytes,blocks", [(4, 12), (400, 12), (4000, 12), (40000, 2)])
def test_reference_shape_benchmark(gpu_built, nbytes, blocks):
    """The reference allocator benchmark's shape (12 x 1024 threads, one
    object each, written, checked and freed; dynamic_allocator/
    benchmarks_template.cu:68-202): every object intact, latencies recorded.
    Objects above 32 KiB are runs of whole pages behind one lock: 2 x 1024
    threads allocate and free them at once."""
    lib = gpu_built.load_library()
    st = gpu_built.malloc_bench(lib, blocks, 1024, nbytes, heap_bytes=1 << 30)
    assert st["allocs"] == st["frees"] == blocks * 1024
    assert st["failed"] == 0 and st["corrupt"] == 0 and st["misaligned"] == 0
    assert 0 < st["malloc_cycles_mean"] and 0 < st["free_cycles_mean"]
    assert st["malloc_cycles_p50"] <= st["malloc_cycles_p99"]
