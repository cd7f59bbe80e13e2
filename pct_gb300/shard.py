"""Sharded DROP over torch.distributed ranks.

The rows of every DROP block are split across ranks (pct_select_shard: rank r
keeps reconstruction histories i with i % world == r) and each block's update
image is summed over the ranks before it is applied (pct_set_allreduce).  The
reference runs every block on one GPU (image_reconstruction_GPU,
src/pCT_Reconstruction_Data_Segments.cu:6803-6844); within a block the rows
are independent given the iterate (block_update_GPU .cu:5774-5841), which is
what makes the split exact up to the order of the float sums.
"""
import ctypes as C

import numpy as np

from . import _capi

_NUMPY = {_capi.PCT_DT_F32: np.float32, _capi.PCT_DT_U32: np.int32, _capi.PCT_DT_F64: np.float64}


def numpy_dtype(dtype):
    """numpy type of a PCT_DT_* buffer (U32 as int32: the same sums bit for bit)."""
    return np.dtype(_NUMPY[dtype])


def host_view(data, count, dtype):
    """numpy view of `count` elements at host address `data`."""
    dt = numpy_dtype(dtype)
    buf = (C.c_char * (int(count) * dt.itemsize)).from_address(data)
    return np.frombuffer(buf, dtype=dt, count=int(count))


class TorchAllReduce:
    """pct_allreduce_fn over a torch.distributed process group.

    Device buffers are staged through a torch tensor on `device` (NCCL sums it
    in place; other backends sum a host copy); host buffers are summed in place.
    Returns non-zero to the library on any failure, which pct_drop reports.
    """

    def __init__(self, group=None, device=None):
        self.group = group
        self.device = device
        self.error = None

    def __call__(self, user, data, count, dtype, on_device):
        try:
            import torch
            import torch.distributed as dist
            if on_device:
                lib = _capi.load()
                tdt = {_capi.PCT_DT_F32: torch.float32, _capi.PCT_DT_U32: torch.int32,
                       _capi.PCT_DT_F64: torch.float64}[dtype]
                t = torch.empty(int(count), dtype=tdt, device=self.device)
                nbytes = t.numel() * t.element_size()
                _capi.check(lib.pct_memcpy(t.data_ptr(), data, nbytes), "pct_memcpy")
                if dist.get_backend(self.group) == "nccl":
                    dist.all_reduce(t, group=self.group)
                else:
                    h = t.cpu()
                    dist.all_reduce(h, group=self.group)
                    t.copy_(h)
                torch.cuda.synchronize(t.device)
                _capi.check(lib.pct_memcpy(data, t.data_ptr(), nbytes), "pct_memcpy")
            else:
                dist.all_reduce(torch.from_numpy(host_view(data, count, dtype)), group=self.group)
            return 0
        except Exception as e:  # reported through the library's status
            self.error = e
            return 1


def shard(recon, rank, world, allreduce):
    """Makes `recon` (after collect_mlp_endpoints) rank `rank` of a `world`-way sharded DROP."""
    recon.select_shard(rank, world)
    recon.set_allreduce(allreduce)
    return recon
