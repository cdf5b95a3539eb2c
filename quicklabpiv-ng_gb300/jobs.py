"""Mirror of the reference's stage-plugin surface for the FFT-PIV path, backed by the
CUDA library.

  Job protocol            S/jobs/Job.java:14-67 (setInputParameters / analyze / compute /
                          getJobResult / dispose)
  xcorr job drop-in       CrossCorrelationRealFFTParStdJob (GPU) / CrossCorrelationSoftRealFFTJob
                          (CPU), created per level by OpenClGpuManager.java:124-140
  shape checks            CrossCorrelationFFTTemplate.analyzeTilesHelper (:594-642)
  results                 XCorrelationResults (S/jobs/xcorr/XCorrelationResults.java:14-55)
  peak + interpolation    IMaximumFinder.findMaximum + ICrossCorrelationInterpolator.interpolate,
                          fused into the kernel (GpuPivStageJob)
(S/ = src/main/java/pt/quickLabPIV/ in QuickLabPIV-ng.)
"""
import enum
from dataclasses import dataclass, field

import numpy as np

from . import (NORM_MAX_A, NORM_OWN_MAX, SUBPIX_GAUSS3, SUBPIX_NONE, SUPPORTED_IA, Handle)


class JobResultEnum(enum.Enum):
    JOB_RESULT_CLIPPED_TILES_A = "JOB_RESULT_CLIPPED_TILES_A"
    JOB_RESULT_CLIPPED_TILES_B = "JOB_RESULT_CLIPPED_TILES_B"
    JOB_RESULT_CROSS_MATRICES = "JOB_RESULT_CROSS_MATRICES"
    JOB_RESULT_CROSS_MAXIMUM = "JOB_RESULT_CROSS_MAXIMUM"


class JobAnalyzeException(RuntimeError):
    pass


class JobComputeException(RuntimeError):
    pass


@dataclass
class Tile:
    """A clipped tile: its pixels (Matrix) and Matrix.getMaxValue()."""
    matrix: np.ndarray
    max_value: float = None
    tile_index_i: int = 0
    tile_index_j: int = 0

    def getMatrix(self):
        return self.matrix


@dataclass
class XCorrelationResults:
    cross_matrices: np.ndarray          # (count, 2N-1, 2N-1) float32
    max_cross_results: list = field(default_factory=list)

    def getCrossMatrices(self):
        return list(self.cross_matrices)

    def getMaxCrossResults(self):
        return self.max_cross_results

    def getDimI(self):
        return self.cross_matrices.shape[1]

    def getDimJ(self):
        return self.cross_matrices.shape[2]

    def getNumberOfMatrices(self):
        return self.cross_matrices.shape[0]


@dataclass
class MaxCrossResult:
    """Main peak of one IA after interpolation (S/maximum/MaxCrossResult.java)."""
    i: float
    j: float
    value: float
    u: float
    v: float
    min_floor: float
    peak_i: int
    peak_j: int
    flags: int

    def getMainPeakI(self):
        return self.i

    def getMainPeakJ(self):
        return self.j

    def getMainPeakValue(self):
        return self.value

    def getNthDisplacementU(self, k=0):
        if k != 0:
            raise IndexError("only the main peak is computed")
        return self.u

    def getNthDisplacementV(self, k=0):
        if k != 0:
            raise IndexError("only the main peak is computed")
        return self.v

    def getMinFloor(self):
        return self.min_floor


class _TileJob:
    """Common Job plumbing for tile-list inputs."""

    def __init__(self, normalization="cpu", device=0, handle=None):
        if normalization not in ("cpu", "gpu"):
            raise ValueError("normalization is 'cpu' (B by A's max) or 'gpu' (own max)")
        self.norm_mode = NORM_MAX_A if normalization == "cpu" else NORM_OWN_MAX
        self._own_handle = handle is None
        self._device = device
        self.handle = handle           # created on first compute()
        self._inputs = {}
        self._results = {}
        self._packed = None

    def setInputParameters(self, key, tiles):
        self._inputs[JobResultEnum(key)] = list(tiles)

    def getJobResult(self, key):
        return self._results.get(JobResultEnum(key))

    def analyze(self):
        tf = self._inputs.get(JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [])
        tg = self._inputs.get(JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, [])
        self._packed = None
        if len(tf) < 1 or len(tg) < 1:
            return
        di, dj = tf[0].matrix.shape
        for t in tf:
            if t.matrix.shape[0] != di:
                raise JobAnalyzeException("Matrices in matricesF don't have the same dimensions (along I)")
            if t.matrix.shape[1] != dj:
                raise JobAnalyzeException("Matrices in matricesF don't have the same dimensions (along J)")
        for t in tg:
            if t.matrix.shape[0] != di:
                raise JobAnalyzeException("Matrices in matricesG don't have the same dimensions (along I)")
            if t.matrix.shape[1] != dj:
                raise JobAnalyzeException("Matrices in matricesG don't have the same dimensions (along J)")
        if di != dj:
            raise JobAnalyzeException("This FFT standard job can only handle square matrices.")
        if len(tf) != len(tg):
            raise JobAnalyzeException("The number of matrices in F must be matched with the number of matrices G")
        if di not in SUPPORTED_IA:
            raise JobAnalyzeException(f"IA size {di} is not supported by the GPU kernels {SUPPORTED_IA}")
        dtype = np.result_type(*[t.matrix.dtype for t in tf + tg])
        if dtype not in (np.uint8, np.uint16, np.float32):
            dtype = np.float32
        ta = np.stack([t.matrix for t in tf]).astype(dtype, copy=False)
        tb = np.stack([t.matrix for t in tg]).astype(dtype, copy=False)
        have_max = all(t.max_value is not None for t in tf + tg)
        ma = np.array([t.max_value for t in tf], np.float32) if have_max else None
        mb = np.array([t.max_value for t in tg], np.float32) if have_max else None
        self._packed = (ta, tb, ma, mb)

    def _handle(self):
        if self.handle is None:
            self.handle = Handle(self._device)
        return self.handle

    def dispose(self):
        if self._own_handle and self.handle is not None:
            self.handle.close()
        self.handle = None


class CrossCorrelationGpuJob(_TileJob):
    """Job<List<Tile>, XCorrelationResults> drop-in: full (2N-1)^2 planes."""

    def compute(self):
        if self._packed is None:
            self._results[JobResultEnum.JOB_RESULT_CROSS_MATRICES] = XCorrelationResults(np.zeros((0, 0, 0), np.float32))
            return
        ta, tb, ma, mb = self._packed
        try:
            planes = self._handle().xcorr_planes(ta, tb, ma, mb, norm_mode=self.norm_mode)
        except RuntimeError as ex:
            raise JobComputeException(str(ex)) from ex
        self._results[JobResultEnum.JOB_RESULT_CROSS_MATRICES] = XCorrelationResults(planes)


class GpuPivStageJob(_TileJob):
    """Fused stage: xcorr + FindMaximumFromCenter + Gaussian1DPolynomial; the plane never
    leaves the GPU.  Result JOB_RESULT_CROSS_MAXIMUM: list of MaxCrossResult."""

    def __init__(self, normalization="cpu", device=0, handle=None, interpolate=True):
        super().__init__(normalization, device, handle)
        self.subpix_mode = SUBPIX_GAUSS3 if interpolate else SUBPIX_NONE

    def compute(self):
        if self._packed is None:
            self._results[JobResultEnum.JOB_RESULT_CROSS_MAXIMUM] = []
            return
        ta, tb, ma, mb = self._packed
        try:
            vec = self._handle().xcorr_peaks(ta, tb, ma, mb, norm_mode=self.norm_mode, subpix_mode=self.subpix_mode)
        except RuntimeError as ex:
            raise JobComputeException(str(ex)) from ex
        self.vectors = vec
        self._results[JobResultEnum.JOB_RESULT_CROSS_MAXIMUM] = [
            MaxCrossResult(float(r["sub_i"]), float(r["sub_j"]), float(r["peak_value"]), float(r["u"]), float(r["v"]),
                           float(r["min_floor"]), int(r["peak_i"]), int(r["peak_j"]), int(r["flags"])) for r in vec]
