"""Precision switches and the mini-batch loader of the reference API
(``qmctorch/utils/torch_utils.py:8-21, 156-207``)."""
from math import ceil

import torch


def set_torch_double_precision():
    torch.set_default_dtype(torch.float64)
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False


def set_torch_single_precision():
    torch.set_default_dtype(torch.float32)
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False


class DataLoader:
    """Mini-batches of walker positions (torch_utils.py:156-207)."""

    def __init__(self, data, batch_size, pin_memory=False):
        self.dataset = data.pin_memory() if (pin_memory and data.device.type == "cpu") else data
        self.len = len(data)
        self.nbatch = ceil(self.len / batch_size)
        self.count = 0
        self.batch_size = batch_size

    def __iter__(self):
        self.count = 0
        return self

    def __next__(self):
        if self.count < self.nbatch - 1:
            out = self.dataset[self.count * self.batch_size:(self.count + 1) * self.batch_size]
            self.count += 1
            return out
        if self.count == self.nbatch - 1:
            out = self.dataset[self.count * self.batch_size:]
            self.count += 1
            return out
        raise StopIteration


from .observable_store import add_group_attr, dump_observables, load_observables  # noqa: E402

__all__ = ["set_torch_double_precision", "set_torch_single_precision", "DataLoader",
           "dump_observables", "add_group_attr", "load_observables"]
