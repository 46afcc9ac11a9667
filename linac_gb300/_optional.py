"""Feature flags, as in linac/_optional.py.

``CUDA_FOUND`` is True when liblinac_gb300.so loads and sees at least one CUDA
device.  The reference also required nvcc on PATH because it compiled its
kernels at run time with pycuda; this build is compiled ahead of time, so only
the library and a device are needed.
"""
try:
    import galois  # noqa: F401
    GALOIS_FOUND = True
except ImportError:
    GALOIS_FOUND = False


def _cuda_is_available() -> bool:
    try:
        from ._lib import device_count
        return device_count() > 0
    except Exception:
        return False


CUDA_FOUND = _cuda_is_available()
