"""ctypes mirrors of the ABI structs in include/lyap_gb300.h.

They reproduce the reference's structs.hpp:20-80 byte for byte (Real = float:
LyapCam/LyapLight 224 B, LyapParams 56 B, LyapPoint 36 B, RGBA 4 B; the *D
classes are the DOUBLE_REALS layouts, 384 / 104 / 72 B).  ctypes cannot
over-align a member, so the 16-byte alignment of the float4/double4 members
(Quat, Color) is spelled out with explicit padding fields named ``_pad*``.
"""
import ctypes
from ctypes import c_float, c_double, c_uint32, c_uint8

import numpy as np

__all__ = [
    "LyapVec", "LyapQuat", "LyapColor", "LyapCam", "LyapLight", "LyapParams",
    "LyapPoint", "RGBA", "LyapVecD", "LyapQuatD", "LyapColorD", "LyapCamD",
    "LyapLightD", "LyapParamsD", "LyapPointD", "POINT_DTYPE", "RGBA_DTYPE",
    "struct_to_bytes", "struct_from_bytes",
]


class _Vec(ctypes.Structure):
    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def __repr__(self):
        return f"{type(self).__name__}({self.x!r}, {self.y!r}, {self.z!r})"


class _Vec4(ctypes.Structure):
    def __iter__(self):
        return iter((self.x, self.y, self.z, self.w))

    def __repr__(self):
        return f"{type(self).__name__}({self.x!r}, {self.y!r}, {self.z!r}, {self.w!r})"


class LyapVec(_Vec):
    """float3 (vec3.hpp VEC3<float, float3>)."""
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]


class LyapQuat(_Vec4):
    """float4 (quat.hpp QUAT<float, float3, float4>); x, y, z vector part, w scalar."""
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("w", c_float)]


class LyapColor(_Vec4):
    """float4 colour (color.hpp COLOR<float, float4>): r, g, b, a in x, y, z, w."""
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("w", c_float)]


class LyapCam(ctypes.Structure):
    """struct _LyapCamLight (structs.hpp:26-51); camera and light share it."""
    _fields_ = [
        ("C", LyapVec), ("_pad0", c_uint8 * 4),
        ("Q", LyapQuat),
        ("M", c_float),
        ("V", LyapVec), ("S0", LyapVec), ("SDX", LyapVec), ("SDY", LyapVec),
        ("textureWidth", c_uint32), ("textureHeight", c_uint32),
        ("renderWidth", c_uint32), ("renderHeight", c_uint32),
        ("renderDenominator", c_uint32),
        ("lightInnerCone", c_float), ("lightOuterCone", c_float),
        ("lightRange", c_float), ("_pad1", c_uint8 * 12),
        ("ambient", LyapColor),
        ("diffuseColor", LyapColor),
        ("diffusePower", c_float), ("_pad2", c_uint8 * 12),
        ("specularColor", LyapColor),
        ("specularPower", c_float), ("specularHardness", c_float),
        ("_pad3", c_uint8 * 8),
        ("chaosColor", LyapColor),
    ]


LyapLight = LyapCam


class LyapParams(ctypes.Structure):
    """LyapParams (structs.hpp:53-68)."""
    _fields_ = [
        ("d", c_float), ("settle", c_uint32), ("accum", c_uint32),
        ("stepMethod", c_uint32), ("nearThreshold", c_float),
        ("nearMultiplier", c_float), ("opaqueThreshold", c_float),
        ("chaosThreshold", c_float), ("depth", c_float), ("jitter", c_float),
        ("refine", c_float), ("gradient", c_float), ("lMin", c_float),
        ("lMax", c_float),
    ]


class LyapPoint(ctypes.Structure):
    """LyapPoint (structs.hpp:70-76)."""
    _fields_ = [("P", LyapVec), ("N", LyapVec), ("a", c_float), ("c", c_float),
                ("l", c_float)]


class RGBA(ctypes.Structure):
    """RGBA (structs.hpp:78-80)."""
    _fields_ = [("r", c_uint8), ("g", c_uint8), ("b", c_uint8), ("a", c_uint8)]


class LyapVecD(_Vec):
    _fields_ = [("x", c_double), ("y", c_double), ("z", c_double)]


class LyapQuatD(_Vec4):
    _fields_ = [("x", c_double), ("y", c_double), ("z", c_double), ("w", c_double)]


class LyapColorD(_Vec4):
    _fields_ = [("x", c_double), ("y", c_double), ("z", c_double), ("w", c_double)]


class LyapCamD(ctypes.Structure):
    """struct _LyapCamLight with Real = double (DOUBLE_REALS)."""
    _fields_ = [
        ("C", LyapVecD), ("_pad0", c_uint8 * 8),
        ("Q", LyapQuatD),
        ("M", c_double),
        ("V", LyapVecD), ("S0", LyapVecD), ("SDX", LyapVecD), ("SDY", LyapVecD),
        ("textureWidth", c_uint32), ("textureHeight", c_uint32),
        ("renderWidth", c_uint32), ("renderHeight", c_uint32),
        ("renderDenominator", c_uint32), ("_pad1", c_uint8 * 4),
        ("lightInnerCone", c_double), ("lightOuterCone", c_double),
        ("lightRange", c_double), ("_pad2", c_uint8 * 8),
        ("ambient", LyapColorD),
        ("diffuseColor", LyapColorD),
        ("diffusePower", c_double), ("_pad3", c_uint8 * 8),
        ("specularColor", LyapColorD),
        ("specularPower", c_double), ("specularHardness", c_double),
        ("chaosColor", LyapColorD),
    ]


LyapLightD = LyapCamD


class LyapParamsD(ctypes.Structure):
    _fields_ = [
        ("d", c_double), ("settle", c_uint32), ("accum", c_uint32),
        ("stepMethod", c_uint32), ("_pad0", c_uint8 * 4),
        ("nearThreshold", c_double), ("nearMultiplier", c_double),
        ("opaqueThreshold", c_double), ("chaosThreshold", c_double),
        ("depth", c_double), ("jitter", c_double), ("refine", c_double),
        ("gradient", c_double), ("lMin", c_double), ("lMax", c_double),
    ]


class LyapPointD(ctypes.Structure):
    _fields_ = [("P", LyapVecD), ("N", LyapVecD), ("a", c_double),
                ("c", c_double), ("l", c_double)]


# numpy views of point / pixel arrays (same bytes as LyapPoint[] / RGBA[])
POINT_DTYPE = np.dtype([("P", "<f4", (3,)), ("N", "<f4", (3,)), ("a", "<f4"),
                        ("c", "<f4"), ("l", "<f4")])
RGBA_DTYPE = np.dtype([("r", "u1"), ("g", "u1"), ("b", "u1"), ("a", "u1")])

assert ctypes.sizeof(LyapCam) == 224 and ctypes.sizeof(LyapParams) == 56
assert ctypes.sizeof(LyapPoint) == 36 and ctypes.sizeof(RGBA) == 4
assert ctypes.sizeof(LyapCamD) == 384 and ctypes.sizeof(LyapParamsD) == 104
assert ctypes.sizeof(LyapPointD) == 72
assert POINT_DTYPE.itemsize == 36


def struct_to_bytes(s):
    return bytes(ctypes.string_at(ctypes.addressof(s), ctypes.sizeof(s)))


def struct_from_bytes(cls, b):
    if len(b) != ctypes.sizeof(cls):
        raise ValueError(f"{cls.__name__} needs {ctypes.sizeof(cls)} bytes, got {len(b)}")
    return cls.from_buffer_copy(b)
