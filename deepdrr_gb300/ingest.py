"""Volume ingest on the GPU (``drr_ingest_hu``): Hounsfield units to densities and material labels
in the projector's texture layout, without the host-side numpy pass of Volume.from_hu
(deepdrr/vol/volume.py:281-351, load_dicom.py:132-143) or a host-to-device copy of its results."""
from __future__ import annotations

import ctypes
from typing import Sequence, Tuple

from . import _lib

_HU_TYPES = {"float32": _lib.DRR_HU_F32, "int16": _lib.DRR_HU_I16, "float64": _lib.DRR_HU_F64}
_DENSITY_TYPES = {"float32": _lib.DRR_DENSITY_F32, "float16": _lib.DRR_DENSITY_F16,
                  "bfloat16": _lib.DRR_DENSITY_BF16}


def hu_to_density_and_labels(hu, density_dtype: str = "float32", class_labels: Sequence[int] = (0, 1, 2),
                             stream=None) -> Tuple["object", "object"]:
    """Densities and labels [nk, nj, ni] (i fastest) from a CUDA tensor of HU [ni, nj, nk].

    ``class_labels`` are the labels of air, soft tissue and bone (default: their ids in
    Volume.from_hu's material dict). float32 HU are converted in float32, int16 / float64 HU in
    float64 (numpy's promotion), then stored as ``density_dtype``."""
    import torch

    if not (isinstance(hu, torch.Tensor) and hu.is_cuda):
        raise TypeError("hu must be a CUDA tensor")
    hu = hu.contiguous()
    name = str(hu.dtype).replace("torch.", "")
    if name not in _HU_TYPES:
        raise TypeError(f"HU dtype {hu.dtype} is not float32, int16 or float64")
    if hu.dim() != 3:
        raise ValueError("hu must be 3D [ni, nj, nk]")
    ni, nj, nk = (int(x) for x in hu.shape)
    tdt = {"float32": torch.float32, "float16": torch.float16, "bfloat16": torch.bfloat16}[density_dtype]
    density = torch.empty((nk, nj, ni), dtype=tdt, device=hu.device)
    labels = torch.empty((nk, nj, ni), dtype=torch.uint8, device=hu.device)
    cls = (ctypes.c_uint8 * 3)(*[int(c) for c in class_labels])
    s = stream if stream is not None else torch.cuda.current_stream(hu.device)
    with torch.cuda.device(hu.device):
        _lib.check(_lib.load().drr_ingest_hu(hu.data_ptr(), _HU_TYPES[name], ni, nj, nk, cls, density.data_ptr(),
                                             _DENSITY_TYPES[density_dtype], labels.data_ptr(),
                                             ctypes.c_void_p(s.cuda_stream)))
    return density, labels
