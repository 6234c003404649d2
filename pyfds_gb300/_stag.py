"""GPU binding shared by the staggered field classes (acoustic and thermal)."""
import numpy as np

from . import _capi
from ._engine import PRECISIONS, StagEngine


class StagField:
    """Mixin: a field whose ``sim_step`` is one fused GPU launch.

    Subclasses set ``_stag_family`` and ``_stag_components`` (potential first, then
    the x and y flux) and implement ``_coefficients()`` returning
    ``(coefs, flags)``: per-cell float64 coefficient arrays keyed like
    ``FdsCoefs`` in include/fds_capi.h and the FDS_FLAG_* bits of the variant.

    Keyword arguments accepted by every constructor on top of the reference's:
      precision: "f64" (default, the drop-in), "f32", "f32_t64" (thermal:
                 float32 fluxes with a float64 temperature) or "dw" (double-word:
                 every value a float32 pair hi + lo with 48-bit significands,
                 compensated float32 arithmetic; float64-class accuracy on the FP32
                 pipe). Thermal "f32" stores the temperature as a
                 deviation from ``potential_offset`` (default: the mean initial
                 temperature); thermal "dw" does so when ``potential_offset`` is set.
      exact:     float64 only; evaluate in the reference's operation order without
                 fused multiply-adds (bit-identical to scipy on x86-64).
      tile:      (x, y) cells per CTA for lossless 2-D fields, one of
                 ``_capi.tile_menu()`` (default: 64 x 16; double words 64 x 12).
    The attribute ``stages`` selects one step per tile (1), the persistent two-stage
    pipeline (2) or two steps per tile and launch (3, lossless 2-D fields); 0 (the
    default) lets the engine choose (two steps per tile for float32 and double-word
    acoustic fields and for batches).
    """

    _stag_family = None
    _stag_components = ()

    def _init_gpu(self, precision="f64", exact=False, tile=None):
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
        if exact and precision != "f64":
            raise ValueError("exact=True requires precision='f64'")
        if precision == "f32_t64" and self._stag_family != _capi.FAMILY_THERMAL:
            raise ValueError("precision='f32_t64' is available for thermal fields only")
        self.precision = precision
        self.exact = bool(exact)
        self.tile = tuple(tile) if tile is not None else None
        # 0: automatic (StagEngine.stages); 1: one step per tile and launch; 2: the
        # persistent two-stage pipeline; 3: two steps per tile (see FdsStagProblem)
        self.stages = 0
        # float32 thermal fields store T - potential_offset (None: the mean initial
        # temperature at the first launch); double-word ones when it is set
        self.potential_offset = None
        self._stag_coefs = None
        self._flags_base = 0
        self._coef_version = 0
        self._eng = None
        self._op_cache = {}

    def _engine(self):
        if self._eng is None:
            self._eng = StagEngine(self)
        return self._eng

    def _stag_flags(self):
        return self._flags_base | (_capi.FLAG_EXACT if self.exact else 0)

    def assemble_matrices(self):
        """Build the per-cell coefficient arrays the kernel reads (the matrix-free
        form of the reference's DIA operators); uploaded on the next launch."""
        coefs, flags = self._coefficients()
        for k in ("by", "ky"):
            base = "bx" if k == "by" else "kx"
            if coefs.get(k) is not None and np.array_equal(coefs[k], coefs[base]):
                coefs[k] = None  # the kernel reads the x array
        self._stag_coefs = coefs
        self._flags_base = flags
        self._coef_version += 1
        self._op_cache = {}
        self.matrices_assembled = True

    def sim_step(self):
        """Simulate one step (``self.step``; ``simulate`` advances the counter)."""
        if not self.matrices_assembled:
            self.assemble_matrices()
        if self._engine().run(self.step, 1, cache_tables=True):
            self._engine().report_nonfinite(self.step + 1)

    _gpu_sim_step = sim_step

    def _operator(self, name, build):
        """Reference-style scipy operator ``a_*`` (None until assembled), for inspection."""
        if not self.matrices_assembled:
            return None
        if name not in self._op_cache:
            self._op_cache[name] = build()
        return self._op_cache[name]

    def __getstate__(self):
        st = self.__dict__.copy()
        st["_eng"] = None
        st["_op_cache"] = {}
        return st


def summed_absorption(nx, has_v, ax, ay, central=None):
    """Diagonals of ``(d_x2(ax) [+ d_y2(ay)] [+ d_x(central, 'central')]).todia()``.

    CSR addition sums coinciding entries left operand first, ``todia`` sorts the
    diagonals by offset (-nx, -1, 0, +1, +nx); for nx == 1 the x and y offsets
    coincide and their values are summed into the x diagonals.
    """
    axm = ax.copy()
    axp = ax.copy()
    if has_v:
        ad = (-2 * ax) + (-2 * ay)
        if nx == 1:
            axm = ax + ay
            axp = ax + ay
            aym = np.zeros_like(ay)
            ayp = np.zeros_like(ay)
        else:
            aym = ay
            ayp = ay
    else:
        ad = -2 * ax
        aym = ayp = None
    if central is not None:
        axm = axm + (-central / 2)
        axp = axp + central / 2
    return {"aym": aym, "axm": axm, "ad": ad, "axp": axp, "ayp": ayp}
