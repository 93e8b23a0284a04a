"""Test helpers: view raw device pointers from the library as torch tensors."""
import numpy as np


class _DevBuf:
    def __init__(self, ptr, nbytes):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def download(ptr, nbytes):
    """Copy nbytes at device address ptr to a numpy array."""
    import torch
    torch.cuda.synchronize()
    t = torch.as_tensor(_DevBuf(ptr, nbytes), device="cuda")
    return t.cpu().numpy().copy()


def padded(frame, pad, stride):
    """frame (H, W) inside a zero buffer with `pad` samples of edge replication, row stride `stride`"""
    H, W = frame.shape
    img = np.zeros((H + 2 * pad, stride), np.uint8)
    img[pad:pad + H, pad:pad + W] = frame
    img[pad:pad + H, :pad] = frame[:, :1]
    img[pad:pad + H, pad + W:pad + W + pad] = frame[:, -1:]
    img[:pad] = img[pad]
    img[pad + H:] = img[pad + H - 1]
    return img.reshape(-1)
