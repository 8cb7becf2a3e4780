"""A GPU-resident mirror of the tmv::Matrix<double> product and division surface.

    A = Matrix(a); B = Matrix(b)
    C = A * B                      # ProdMM -> MultMM<false>  (TMV_MatrixArith.h:701-730)
    A.divideUsing(LU); A.saveDiv() # DivHelper flags          (src/TMV_BaseMatrix.cpp:215-223)
    X = B / A                      # QuotMM -> LUDiv::doLDiv  (TMV_MatrixArith.h:1145-1175)
    Y = W % A                      # RQuotMM -> LUDiv::doRDiv (TMV_MatrixArith.h:1197-1227)
    A.det(), A.logDet(), A.lud().getP(), A.isSingular()

Storage is column-major float64 on the current CUDA device.  As in TMV, the
LU divider is created lazily on the first division and destroyed after it
unless saveDiv() was called (src/TMV_BaseMatrix.cpp:170-190, 273-274).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import linalg

LU = "LU"
ColMajor = "ColMajor"
RowMajor = "RowMajor"


class LUDiv:
    """The LU decomposition of a matrix (tmv::LUDiv<double>, include/tmv/TMV_LUD.h:90-161)."""

    def __init__(self, m: "Matrix", inplace: bool = False):
        src = m.t
        if inplace:
            self.LU = src
        else:
            self.LU = torch.empty_like(src.t()).t()
            self.LU.copy_(src)
        self.P = linalg.lu_decompose(self.LU)
        self._det = None

    def isTrans(self) -> bool:
        return False

    def getLU(self) -> torch.Tensor:
        return self.LU

    def getL(self) -> torch.Tensor:
        n = self.LU.shape[0]
        return torch.tril(self.LU, -1) + torch.eye(n, dtype=self.LU.dtype, device=self.LU.device)

    def getU(self) -> torch.Tensor:
        return torch.triu(self.LU)

    def getP(self) -> np.ndarray:
        return self.P.cpu().numpy()

    def det(self) -> float:
        if self._det is None:
            self._det = linalg.lu_det(self.LU, self.P)
        return self._det[0]

    def logDet(self):
        if self._det is None:
            self._det = linalg.lu_det(self.LU, self.P)
        return self._det[1], self._det[2]

    def isSingular(self) -> bool:
        return linalg.lu_is_singular(self.LU)

    def makeInverse(self) -> torch.Tensor:
        """A^-1 (LUDiv::doMakeInverse, src/TMV_LUD.cpp:158-170)."""
        return linalg.lu_inverse(self.LU, self.P)

    def makeInverseATA(self) -> torch.Tensor:
        """(A^T A)^-1 (LUDiv::doMakeInverseATA, src/TMV_LUD.cpp:172-200)."""
        return linalg.lu_inverse_ata(self.LU)

    def ldiv(self, b: torch.Tensor) -> torch.Tensor:
        x = linalg.colmajor(b)
        linalg.lu_ldiveq(self.LU, self.P, x)
        return x

    def rdiv(self, b: torch.Tensor) -> torch.Tensor:
        x = linalg.colmajor(b)
        linalg.lu_rdiveq(self.LU, self.P, x)
        return x


UnitDiag = "UnitDiag"
NonUnitDiag = "NonUnitDiag"


class TriMatrixView:
    """The upper or lower triangle of a Matrix (m.upperTri(dt), m.lowerTri(dt):
    tmv::UpperTriMatrixView / LowerTriMatrixView).  `B / T` is T^-1 B and
    `B % T` is B T^-1 (TriLDivEq, src/TMV_TriDiv_M.cpp:583-710)."""

    def __init__(self, t: torch.Tensor, upper: bool, dt: str):
        if dt not in (UnitDiag, NonUnitDiag):
            raise ValueError("dt must be UnitDiag or NonUnitDiag")
        self.t = t
        self.upper = upper
        self.unit = dt == UnitDiag

    def size(self) -> int:
        return self.t.shape[0]


class Matrix:
    """Column-major float64 matrix on a CUDA device (tmv::Matrix<double,ColMajor>)."""

    def __init__(self, data, device=None):
        if isinstance(data, Matrix):
            data = data.t
        if isinstance(data, torch.Tensor):
            t = data.to(dtype=torch.float64, device=device or data.device if data.is_cuda else "cuda")
        else:
            a = np.asarray(data, dtype=np.float64)
            t = torch.from_numpy(a).to(device or "cuda")
        if t.dim() == 1:
            t = t.view(-1, 1)
        self.t = linalg.colmajor(t)
        self._divtype = None
        self._savediv = False
        self._inplace = False
        self._div: LUDiv | None = None

    # -- shape -------------------------------------------------------------
    def colsize(self) -> int:
        return self.t.shape[0]

    def rowsize(self) -> int:
        return self.t.shape[1]

    @property
    def shape(self):
        return tuple(self.t.shape)

    def numpy(self) -> np.ndarray:
        return self.t.cpu().numpy()

    def upperTri(self, dt: str = NonUnitDiag) -> TriMatrixView:
        return TriMatrixView(self.t, True, dt)

    def lowerTri(self, dt: str = NonUnitDiag) -> TriMatrixView:
        return TriMatrixView(self.t, False, dt)

    # -- product -----------------------------------------------------------
    def __mul__(self, other):
        if isinstance(other, (int, float)):
            return Matrix(self.t * float(other))
        if (isinstance(other, torch.Tensor) or isinstance(other, np.ndarray)) and other.ndim == 1:
            # y = A x (MultMV<false>, src/TMV_MultMV.cpp:1134)
            x = torch.as_tensor(other, dtype=torch.float64, device=self.t.device)
            y = torch.empty(self.colsize(), dtype=torch.float64, device=self.t.device)
            linalg.multmv(False, 1.0, self.t, x, y)
            return y
        if not isinstance(other, Matrix):
            other = Matrix(other)
        m, k = self.shape
        k2, n = other.shape
        if k != k2:
            raise ValueError("size mismatch in product")
        out = torch.empty((n, m), dtype=torch.float64, device=self.t.device).t()
        linalg.multmm(False, 1.0, self.t, other.t, out)
        return Matrix._wrap(out)

    __matmul__ = __mul__

    @staticmethod
    def _wrap(t: torch.Tensor) -> "Matrix":
        m = Matrix.__new__(Matrix)
        m.t = t
        m._divtype = None
        m._savediv = False
        m._inplace = False
        m._div = None
        return m

    # -- division control (DivHelper) ---------------------------------------
    def divideUsing(self, dt) -> None:
        if dt != LU:
            raise NotImplementedError("only tmv::LU is implemented on the GPU")
        if self._divtype != dt:
            self._div = None
        self._divtype = dt

    def saveDiv(self) -> None:
        self._savediv = True

    def divideInPlace(self) -> None:
        self._inplace = True
        self._savediv = True

    def setDiv(self) -> None:
        if self._div is None:
            if self.colsize() != self.rowsize():
                raise NotImplementedError("LU division of non-square matrices is out of scope")
            self._divtype = self._divtype or LU
            self._div = LUDiv(self, self._inplace)

    def unsetDiv(self) -> None:
        self._div = None

    def resetDiv(self) -> None:
        self.unsetDiv()
        self.setDiv()

    def lud(self) -> LUDiv:
        self.divideUsing(LU)
        self.setDiv()
        return self._div

    def _done(self) -> None:
        if not self._savediv:
            self._div = None

    def _ldiv(self, b: "Matrix") -> "Matrix":
        self.setDiv()
        x = self._div.ldiv(b.t)
        self._done()
        return Matrix._wrap(x)

    def _rdiv(self, b: "Matrix") -> "Matrix":
        self.setDiv()
        bt = b.t if b.t.shape[1] == self.colsize() else b.t.t()
        x = self._div.rdiv(bt)
        self._done()
        return Matrix._wrap(x)

    def __truediv__(self, other):
        """self / other: for a Matrix `other`, X = other^-1 self (TMV's b/m);
        for a triangle, X = T^-1 self (TriLDivEq)."""
        if isinstance(other, (int, float)):
            return Matrix(self.t / float(other))
        if isinstance(other, TriMatrixView):
            x = linalg.colmajor(self.t)
            linalg.tri_ldiveq(other.t, other.upper, other.unit, x)
            return Matrix._wrap(x)
        if not isinstance(other, Matrix):
            other = Matrix(other)
        return other._ldiv(self)

    def __mod__(self, other):
        """self % other: X = self other^-1 (TMV's b%m); X = self T^-1 for a triangle."""
        if isinstance(other, TriMatrixView):
            x = linalg.colmajor(self.t)
            linalg.tri_rdiveq(other.t, other.upper, other.unit, x)
            return Matrix._wrap(x)
        if not isinstance(other, Matrix):
            other = Matrix(other)
        return other._rdiv(self)

    # -- decomposition queries ------------------------------------------------
    def det(self) -> float:
        self.setDiv()
        d = self._div.det()
        self._done()
        return d

    def logDet(self):
        self.setDiv()
        r = self._div.logDet()
        self._done()
        return r

    def isSingular(self) -> bool:
        self.setDiv()
        r = self._div.isSingular()
        self._done()
        return r

    def inverse(self) -> "Matrix":
        self.setDiv()
        r = Matrix._wrap(self._div.makeInverse())
        self._done()
        return r

    def makeInverseATA(self) -> "Matrix":
        self.setDiv()
        r = Matrix._wrap(self._div.makeInverseATA())
        self._done()
        return r

    def norm(self) -> float:
        return float(torch.linalg.norm(self.t))


def Norm(m: Matrix) -> float:
    return m.norm() if isinstance(m, Matrix) else float(np.linalg.norm(m))


__all__ = ["Matrix", "LUDiv", "LU", "ColMajor", "RowMajor", "Norm", "math"]
