"""Device columns (gdf_column) and scalars (gdf_scalar) for the C ABI."""
from __future__ import annotations

import ctypes
import struct
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import dtypes as D


class GdfDtypeExtraInfo(ctypes.Structure):
    _fields_ = [("time_unit", ctypes.c_int32), ("category", ctypes.c_void_p)]


class GdfColumn(ctypes.Structure):
    """struct gdf_column_ of include/ral/gdf_compat.h."""
    _fields_ = [("data", ctypes.c_void_p), ("valid", ctypes.c_void_p), ("size", ctypes.c_int32),
                ("dtype", ctypes.c_int32), ("null_count", ctypes.c_int32),
                ("dtype_info", GdfDtypeExtraInfo), ("col_name", ctypes.c_char_p)]


class GdfScalar(ctypes.Structure):
    """gdf_scalar {gdf_data data; gdf_dtype dtype; bool is_valid;}."""
    _fields_ = [("data", ctypes.c_uint64), ("dtype", ctypes.c_int32), ("is_valid", ctypes.c_bool)]


def valid_alloc_size(n: int) -> int:
    """gdf_valid_allocation_size: bytes for n bits, padded to 64 bytes."""
    return ((n + 7) // 8 + 63) // 64 * 64


@dataclass
class Scalar:
    dtype: int
    value: float | int = 0
    is_valid: bool = True

    def raw(self) -> int:
        t = self.dtype
        if t == D.GDF_FLOAT32:
            b = struct.pack("<f", float(self.value)) + b"\0" * 4
        elif t == D.GDF_FLOAT64:
            b = struct.pack("<d", float(self.value))
        elif t in (D.GDF_INT8, D.GDF_BOOL8):
            b = struct.pack("<b", int(self.value)) + b"\0" * 7
        elif t == D.GDF_INT16:
            b = struct.pack("<h", int(self.value)) + b"\0" * 6
        elif t in (D.GDF_INT32, D.GDF_DATE32, D.GDF_STRING_CATEGORY):
            b = struct.pack("<i", int(self.value)) + b"\0" * 4
        else:
            b = struct.pack("<q", int(self.value))
        return struct.unpack("<Q", b)[0]

    def to_c(self) -> GdfScalar:
        return GdfScalar(self.raw(), self.dtype, bool(self.is_valid))

    @staticmethod
    def from_c(s: GdfScalar) -> "Scalar":
        raw = struct.pack("<Q", s.data)
        t = s.dtype
        if t == D.GDF_FLOAT32:
            v = struct.unpack("<f", raw[:4])[0]
        elif t == D.GDF_FLOAT64:
            v = struct.unpack("<d", raw)[0]
        elif t in (D.GDF_INT8, D.GDF_BOOL8):
            v = struct.unpack("<b", raw[:1])[0]
        elif t == D.GDF_INT16:
            v = struct.unpack("<h", raw[:2])[0]
        elif t in (D.GDF_INT32, D.GDF_DATE32, D.GDF_STRING_CATEGORY):
            v = struct.unpack("<i", raw[:4])[0]
        else:
            v = struct.unpack("<q", raw)[0]
        return Scalar(t, v, bool(s.is_valid))


class Column:
    """A device column: data tensor (size elements), optional padded validity
    tensor (uint8, valid_alloc_size(capacity) bytes), dtype, null_count."""

    def __init__(self, data, valid, dtype: int, size: Optional[int] = None, null_count: int = 0,
                 category: Optional[int] = None):
        self.data = data
        self.valid = valid
        self.dtype = dtype
        self.size = int(data.shape[0]) if size is None else int(size)
        self.null_count = int(null_count)
        self.category = category   # GDF_STRING_CATEGORY: address of the ral_category dictionary
        self._c: Optional[GdfColumn] = None

    # -- construction -------------------------------------------------------------------------
    @staticmethod
    def empty(dtype: int, n: int, with_valid: bool = True, device="cuda", fill_valid: int = 0xFF) -> "Column":
        import torch
        data = torch.empty(max(n, 1), dtype=D.torch_dtype(dtype), device=device)
        valid = None
        if with_valid:
            valid = torch.full((valid_alloc_size(max(n, 1)),), fill_valid, dtype=torch.uint8, device=device)
        return Column(data, valid, dtype, size=n)

    @staticmethod
    def from_numpy(values, dtype: int, valids=None, null_count: Optional[int] = None, device="cuda") -> "Column":
        import torch
        arr = np.ascontiguousarray(np.asarray(values).astype(D.NP[dtype]))
        n = arr.shape[0]
        data = torch.from_numpy(arr.copy() if n else np.zeros(1, dtype=D.NP[dtype])).to(device)
        valid = None
        nc = 0
        if valids is not None:
            vb = np.asarray(valids, dtype=bool)
            buf = np.zeros(valid_alloc_size(max(n, 1)), dtype=np.uint8)
            packed = np.packbits(vb[:n], bitorder="little")
            buf[:len(packed)] = packed
            valid = torch.from_numpy(buf).to(device)
            nc = int((~vb[:n]).sum()) if null_count is None else null_count
        return Column(data, valid, dtype, size=n, null_count=nc)

    @staticmethod
    def from_valid_bytes(values, dtype: int, valid_bytes: Optional[np.ndarray], null_count: int,
                         device="cuda") -> "Column":
        import torch
        arr = np.ascontiguousarray(np.asarray(values).astype(D.NP[dtype]))
        n = arr.shape[0]
        data = torch.from_numpy(arr.copy() if n else np.zeros(1, dtype=D.NP[dtype])).to(device)
        valid = None if valid_bytes is None else torch.from_numpy(np.ascontiguousarray(valid_bytes)).to(device)
        return Column(data, valid, dtype, size=n, null_count=null_count)

    # -- views ----------------------------------------------------------------------------------
    def to_numpy(self) -> np.ndarray:
        return self.data[:self.size].cpu().numpy()

    def valid_bools(self) -> np.ndarray:
        if self.valid is None:
            return np.ones(self.size, dtype=bool)
        return np.unpackbits(self.valid.cpu().numpy(), bitorder="little")[:self.size].astype(bool)

    def valid_bytes(self) -> Optional[np.ndarray]:
        return None if self.valid is None else self.valid.cpu().numpy()

    # -- C interop ------------------------------------------------------------------------------
    def to_c(self) -> GdfColumn:
        c = GdfColumn()
        c.data = self.data.data_ptr() if self.data is not None else None
        c.valid = self.valid.data_ptr() if self.valid is not None else None
        c.size = self.size
        c.dtype = self.dtype
        c.null_count = self.null_count
        if self.category:
            c.dtype_info.category = self.category
        self._c = c
        return c

    def sync_from_c(self, c: GdfColumn) -> None:
        self.size = int(c.size)
        self.null_count = int(c.null_count)
        if c.dtype_info.category:
            self.category = int(c.dtype_info.category)

    def __repr__(self):
        return f"Column({D.NAMES.get(self.dtype, self.dtype)}, size={self.size}, nulls={self.null_count})"
