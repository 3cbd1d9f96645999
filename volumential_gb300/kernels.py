"""Integral kernel descriptors.

The reference passes sumpy kernel objects (``sumpy.kernel.LaplaceKernel``,
``HelmholtzKernel``, ``AxisTargetDerivative`` ...) and the table manager's
``ConstantKernel`` (``volumential/table_manager.py:360-385``).  sumpy is not a
dependency here, so these light classes carry what the list-1 path reads:
``dim``, ``is_complex_valued``, ``repr`` (the kernel name used in cache keys
and for the ``CstKnl2D``-style checks of ``list1.py:238-242``),
``get_base_kernel()`` and ``inner_kernel``.  Every check in this package is by
class name, so genuine sumpy kernel objects are accepted as well.
"""

from __future__ import annotations

import math

import numpy as np

__all__ = [
    "LaplaceKernel", "HelmholtzKernel", "YukawaKernel", "ConstantKernel",
    "AxisTargetDerivative", "AxisSourceDerivative", "RadialPowerKernel",
    "RadialPowerLogKernel", "PlaneWaveKernel", "arithmetic_symmetry", "base_kernel",
    "kernel_class_name", "green_function_constants",
]


class _Kernel:
    is_complex_valued = False
    # invariant under the box's axis permutations and reflections (the
    # arithmetic orbit reconstruction); kernels that are not keep full tables
    # and the dense reconstruction
    has_orbit_symmetry = True

    def get_base_kernel(self):
        return self

    def __eq__(self, other):
        return type(self) is type(other) and repr(self) == repr(other)

    def __hash__(self):
        return hash(repr(self))


class LaplaceKernel(_Kernel):
    """Free-space Laplace Green's function: -log(r)/(2 pi) in 2D, 1/(4 pi r) in 3D."""

    def __init__(self, dim):
        self.dim = int(dim)

    def __repr__(self):
        return f"LapKnl{self.dim}D"


class HelmholtzKernel(_Kernel):
    """(i/4) H0(1)(k r) in 2D, exp(i k r)/(4 pi r) in 3D."""

    is_complex_valued = True

    def __init__(self, dim, helmholtz_k_name="k", allow_evanescent=False):
        self.dim = int(dim)
        self.helmholtz_k_name = helmholtz_k_name
        self.allow_evanescent = allow_evanescent

    def __repr__(self):
        return f"HelmKnl{self.dim}D({self.helmholtz_k_name})"


class YukawaKernel(_Kernel):
    def __init__(self, dim, yukawa_lambda_name="lam"):
        self.dim = int(dim)
        self.yukawa_lambda_name = yukawa_lambda_name

    def __repr__(self):
        return f"YukKnl{self.dim}D({self.yukawa_lambda_name})"


class ConstantKernel(_Kernel):
    """K = 1 (``volumential/table_manager.py:360-385``)."""

    def __init__(self, dim=None):
        self.dim = int(dim)

    def __repr__(self):
        return "CstKnl%dD" % self.dim


class RadialPowerKernel(_Kernel):
    """K = r^power (scaling constant 1): the 3D Helmholtz split mode's extra
    term kernels (``volumential/expansion_wrangler_fpnd.py:144-175``)."""

    def __init__(self, dim, power):
        if int(power) < 0:
            raise ValueError("power must be non-negative")
        self.dim = int(dim)
        self.power = int(power)

    def __repr__(self):
        return f"RadialPowerKernel(dim={self.dim}, power={self.power})"


class RadialPowerLogKernel(_Kernel):
    """K = r^power log r (scaling constant 1): the 2D Helmholtz split mode's
    extra term kernels (``volumential/expansion_wrangler_fpnd.py:178-209``)."""

    def __init__(self, dim, power):
        if int(power) <= 0:
            raise ValueError("power must be positive for r**power * log(r)")
        self.dim = int(dim)
        self.power = int(power)

    def __repr__(self):
        return f"RadialPowerLogKernel(dim={self.dim}, power={self.power})"


class PlaneWaveKernel(_Kernel):
    """K = cos(k d_0) (scaling constant 1), the plane wave of the reference's
    manufactured Duffy tests (``test/test_duffy_batched_manufactured.py:
    219-284``).  It is not invariant under axis permutations, so its tables
    are full and take the dense reconstruction."""

    has_orbit_symmetry = False

    def __init__(self, dim, plane_wave_k_name="k"):
        self.dim = int(dim)
        self.plane_wave_k_name = plane_wave_k_name

    def __repr__(self):
        return f"PlaneWaveKnl{self.dim}D({self.plane_wave_k_name})"


class _Derivative(_Kernel):
    def __init__(self, axis, inner_kernel):
        self.axis = int(axis)
        self.inner_kernel = inner_kernel
        self.dim = inner_kernel.dim

    @property
    def is_complex_valued(self):
        return self.inner_kernel.is_complex_valued

    def get_base_kernel(self):
        return self.inner_kernel.get_base_kernel()


class AxisTargetDerivative(_Derivative):
    def __repr__(self):
        return f"AxisTargetDerivative({self.axis}, {self.inner_kernel!r})"


class AxisSourceDerivative(_Derivative):
    def __repr__(self):
        return f"AxisSourceDerivative({self.axis}, {self.inner_kernel!r})"


def arithmetic_symmetry(knl, dim):
    """The arithmetic orbit symmetry of a derivative chain over an
    orbit-symmetric kernel (``volumential/orbit_arithmetic.py:176-300``):
    each differentiated axis is fixed (its own axis group) and odd under
    reflection (sign power XOR 1 per derivative), the other axes form one
    permutable group.  ``None`` for an undifferentiated kernel (the scalar
    symmetry); ``False`` when the chain has no arithmetic symmetry."""
    dim = int(dim)
    fixed = set()
    sign_power = np.zeros(dim, dtype=np.uint8)
    k = knl
    while k is not None:
        name = type(k).__name__
        if name in ("AxisTargetDerivative", "AxisSourceDerivative"):
            axis = int(k.axis)
            if not 0 <= axis < dim:
                return False
            fixed.add(axis)
            sign_power[axis] ^= 1
            k = k.inner_kernel
            continue
        if hasattr(k, "inner_kernel"):
            return False   # other wrappers (directional derivatives) are not built
        break
    if not getattr(k, "has_orbit_symmetry", True):
        return False
    if not fixed:
        return None
    free = tuple(a for a in range(dim) if a not in fixed)
    groups = tuple((a,) for a in sorted(fixed)) + ((free,) if free else ())
    return {"axis_groups": groups, "axis_sign_power": sign_power,
            "axis_direction_signs": np.zeros(dim, dtype=np.int8),
            "direction_sign_axis": -1}


def base_kernel(knl):
    get = getattr(knl, "get_base_kernel", None)
    return get() if get is not None else knl


def kernel_class_name(knl):
    return type(knl).__name__


def green_function_constants(knl):
    """(name, dim) of the base Green's function, for table builders."""
    b = base_kernel(knl)
    return kernel_class_name(b), int(b.dim)


LAPLACE_2D_COEF = -0.5 / math.pi
