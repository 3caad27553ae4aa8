"""Device plumbing: PyTorch provides device memory and streams; the compute
runs in libsucem_gb300.so.  There is no CPU fallback."""
import torch

_DEVICE = None


def device():
    """The CUDA device the GPU path uses (cuda:0 unless set_device was called)."""
    global _DEVICE
    if _DEVICE is None:
        if not torch.cuda.is_available():
            raise RuntimeError("sucemfem GB300 path needs a CUDA device; none is visible")
        _DEVICE = torch.device("cuda", torch.cuda.current_device())
    return _DEVICE


def set_device(index):
    global _DEVICE
    torch.cuda.set_device(index)
    _DEVICE = torch.device("cuda", index)


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream(device())
    return s.cuda_stream


def empty(n, dtype):
    return torch.empty(int(n), dtype=dtype, device=device())


def to_dev(a, dtype=None):
    t = torch.as_tensor(a)
    if dtype is not None:
        t = t.to(dtype)
    return t.to(device(), non_blocking=False).contiguous()


REAL = {4: torch.float32, 8: torch.float64}
COMPLEX = {4: torch.complex64, 8: torch.complex128}
