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

__all__ = [
    "LaplaceKernel", "HelmholtzKernel", "YukawaKernel", "ConstantKernel",
    "AxisTargetDerivative", "AxisSourceDerivative", "RadialPowerKernel",
    "RadialPowerLogKernel", "base_kernel",
    "kernel_class_name", "green_function_constants",
]


class _Kernel:
    is_complex_valued = False

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
