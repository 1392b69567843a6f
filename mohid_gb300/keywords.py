"""MOHID keyword data files and the advection-diffusion options they give each
property of a WaterProperties file.

A MOHID data file (read by ModuleEnterData, Software/MOHIDBase1/ModuleEnterData.F90)
is a list of `KEYWORD : value` lines, grouped into blocks such as
`<beginproperty>` ... `<endproperty>`:

* everything from a `!` to the end of the line is a comment, tabs count as
  spaces and lines are read left-adjusted (ConstructEnterData, :300-330);
* the keyword is the text before the first `:` (trailing blanks dropped); when
  the `:` is followed by `/` or `\\` (a drive letter, `C:\\...`) the first blank
  delimits instead, and a line whose keyword matches without a `:` is an error
  (ScanLine :1326-1370, LookForLineInBlock :1180-1267); matching is case
  sensitive;
* a search from the file takes the first matching line anywhere in the file,
  a search from a block the first inside the block;
* reals and integers are read list-directed from the text after the delimiter
  (`1.e-8`, `1.0d0`); a logical is the integer 0 or 1, and a matching line with
  nothing readable counts as 1 (ReadLogical_New :1941-2122).

`property_options` restates Read_Advec_Difus_Parameters
(Software/MOHIDWater/ModuleWaterProperties.F90:9226-9733), which reads each
property's options: the horizontal and vertical methods, limiters and
VOLUME_RELATION_MAX from the file, the rest from the property's block, with
the reference's defaults; the *_IMP_EXP keywords give the explicit weight,
the step's the implicit one (1 - value).  ADVECTION_DIFFUSION (:8255, default
1) and DISCHARGES say whether the property is transported and has point
sources.
"""
from __future__ import annotations

import dataclasses
import re
from pathlib import Path

__all__ = ["KeywordError", "EnterData", "PropertyOptions", "property_options", "step_directions", "BatchPlan",
           "batch_plan"]


class KeywordError(ValueError):
    """A data file the reference stops on (invalid delimiter, logical not 0/1,
    a value it cannot read, an option combination it rejects)."""


@dataclasses.dataclass
class _Line:
    text: str
    number: int


class EnterData:
    """The lines of one keyword data file, as ModuleEnterData buffers them."""

    def __init__(self, text: str, name: str = "<text>"):
        self.name = name
        self.lines: list[_Line] = []
        for n, raw in enumerate(text.splitlines(), 1):
            line = raw.lstrip().replace("\t", " ")
            cut = line.find("!")
            if cut >= 0:
                line = line[:cut]
            self.lines.append(_Line(line.rstrip(), n))

    @classmethod
    def from_file(cls, path) -> "EnterData":
        p = Path(path)
        return cls(p.read_bytes().decode("latin-1"), str(p))

    # -- blocks -------------------------------------------------------------
    def blocks(self, begin: str = "<beginproperty>", end: str = "<endproperty>") -> list[tuple[int, int]]:
        """(first, last) line indices of each block's body, in file order."""
        out, start = [], None
        for q, ln in enumerate(self.lines):
            word = ln.text.strip()
            if word == begin:
                if start is not None:
                    raise KeywordError(f"{self.name}:{ln.number}: {begin} inside an open block")
                start = q + 1
            elif word == end:
                if start is None:
                    raise KeywordError(f"{self.name}:{ln.number}: {end} without {begin}")
                out.append((start, q - 1))
                start = None
        if start is not None:
            raise KeywordError(f"{self.name}: {begin} without {end}")
        return out

    # -- keyword lookup -----------------------------------------------------
    @staticmethod
    def _split(text: str) -> tuple[str, str, bool]:
        """(keyword, value text, valid delimiter) of one line."""
        pos = text.find(":")
        valid = True
        if pos < 0:
            pos, valid = text.find(" "), False
        elif pos + 1 < len(text) and text[pos + 1] in "/\\":
            pos = text.find(" ")
        if pos < 0:
            return text.rstrip(), "", valid
        return text[:pos].rstrip(), text[pos + 1:], valid

    def find(self, keyword: str, block: tuple[int, int] | None = None) -> _Line | None:
        lo, hi = (0, len(self.lines) - 1) if block is None else block
        for ln in self.lines[lo:hi + 1]:
            key, _, valid = self._split(ln.text)
            if key == keyword:
                if not valid:
                    raise KeywordError(f"{self.name}:{ln.number}: invalid delimiter between keyword and value")
                return ln
        return None

    def _value(self, keyword, block):
        ln = self.find(keyword, block)
        if ln is None:
            return None, None
        return self._split(ln.text)[1], ln

    @staticmethod
    def _first_token(text: str) -> str:
        tok = re.split(r"[\s,]+", text.strip(), maxsplit=1)
        return tok[0] if tok and tok[0] else ""

    def real(self, keyword: str, default: float, block=None) -> float:
        text, ln = self._value(keyword, block)
        if text is None:
            return default
        tok = self._first_token(text).replace("d", "e").replace("D", "e")
        try:
            return float(tok)
        except ValueError:
            raise KeywordError(f"{self.name}:{ln.number}: {keyword}: cannot read a real from {text.strip()!r}")

    def integer(self, keyword: str, default: int, block=None) -> int:
        text, ln = self._value(keyword, block)
        if text is None:
            return default
        try:
            return int(self._first_token(text))
        except ValueError:
            raise KeywordError(f"{self.name}:{ln.number}: {keyword}: cannot read an integer from {text.strip()!r}")

    def logical(self, keyword: str, default: bool, block=None) -> bool:
        text, ln = self._value(keyword, block)
        if text is None:
            return default
        try:
            v = int(self._first_token(text))
        except ValueError:
            v = 1                                   # nothing readable counts as 1
        if v not in (0, 1):
            raise KeywordError(f"{self.name}:{ln.number}: value in front of a logical keyword must be 0 or 1")
        return v == 1

    def string(self, keyword: str, default: str = "", block=None) -> str:
        text, _ = self._value(keyword, block)
        return default if text is None else text.strip()


# option codes (ModuleGlobalData.F90:1810-1811, ModuleAdvectionDiffusion.F90:861-880)
_UPWIND2_METHODS = (2, 3, 4)                    # UpwindOrder2, UpwindOrder3, P2_TVD
_BOUNDARY_CONDITIONS = (1, 2, 4, 5, 6, 7, 8)


@dataclasses.dataclass
class PropertyOptions:
    """The advection-diffusion options of one property block."""
    name: str
    advection_diffusion: bool
    discharges: bool
    implicit_h: bool            # horizontal advection implicit, alternating j / i direction each step
    params: dict                # mohid_ad_params fields (advdiff.params keywords), DTProp excluded


def property_options(data: EnterData, block: tuple[int, int]) -> PropertyOptions:
    """Read_Advec_Difus_Parameters (ModuleWaterProperties.F90:9226-9733) for one
    property block: the mohid_ad_params a WaterProperties file gives it."""
    g = data
    p = dict(
        schmidt_H=g.real("SCHMIDT_NUMBER_H", 1.0, block),
        SchmidtCoef_V=g.real("SCHMIDT_COEF_V", 1.0, block),
        SchmidtBackground_V=g.real("SCHMIDT_BACKGROUND_V", 1.0e-8, block),
        ImpExp_AdvV=1.0 - g.real("ADVECTION_V_IMP_EXP", 0.0, block),
        ImpExp_DifV=1.0 - g.real("DIFFUSION_V_IMP_EXP", 0.0, block),
        NullDif=int(g.logical("NULLDIF", False, block)),
        DecayTime=g.real("DECAY_TIME", 0.0, block),
    )
    bc = g.integer("BOUNDARY_CONDITION", 1, block)
    if bc not in _BOUNDARY_CONDITIONS:
        raise KeywordError(f"{data.name}: BOUNDARY_CONDITION {bc} (reference ERR100)")
    p["BoundaryCondition"] = bc
    adv_h = 1.0 - g.real("ADVECTION_H_IMP_EXP", 1.0, block)
    p["ImpExp_DifH"] = 0.0
    # the methods, limiters and volume ratio are read from the whole file
    mh, mv = g.integer("ADV_METHOD_H", 1), g.integer("ADV_METHOD_V", 1)
    p.update(AdvMethodH=mh, TVDLimitationH=g.integer("TVD_LIMIT_H", 4), AdvMethodV=mv,
             TVDLimitationV=g.integer("TVD_LIMIT_V", 4), VolumeRelMax=g.real("VOLUME_RELATION_MAX", 1.5))
    p["Upwind2H"] = int(mh in _UPWIND2_METHODS)
    p["Upwind2V"] = int(mv in _UPWIND2_METHODS)
    if adv_h > 0.0 and mh in (2, 3):
        raise KeywordError(f"{data.name}: implicit horizontal advection with a second or third order "
                           "upwind method (reference ERR190)")
    if p["ImpExp_AdvV"] > 0.0 and mv in (2, 3):
        raise KeywordError(f"{data.name}: implicit vertical advection with a second or third order "
                           "upwind method (reference ERR200)")
    nudging = g.logical("ADVECTION_NUDGING", False, block)
    p["AdvectionNudging"] = int(nudging)
    p["AdvectionNudgingCells"] = g.integer("ADVECTION_NUDGING_CELLS", 10, block) if nudging else 0
    return PropertyOptions(name=g.string("NAME", "", block),
                           advection_diffusion=g.logical("ADVECTION_DIFFUSION", True, block),
                           discharges=g.logical("DISCHARGES", False, block),
                           implicit_h=adv_h == 1.0, params=p)


def step_directions(opt: PropertyOptions, step: int) -> dict:
    """ImpExp_AdvXX / ImpExp_AdvYY of the property's step number `step` (0 first):
    with implicit horizontal advection the implicit direction alternates, j
    (XX) first (ModuleWaterProperties.F90:14681-14707)."""
    if not opt.implicit_h:
        return dict(ImpExp_AdvXX=0.0, ImpExp_AdvYY=0.0)
    x = step % 2 == 0
    return dict(ImpExp_AdvXX=1.0 if x else 0.0, ImpExp_AdvYY=0.0 if x else 1.0)


@dataclasses.dataclass
class BatchPlan:
    """How the transported properties of a WaterProperties file map onto the
    library: groups of properties that share every option go through one
    batched call each (mohid_ad_batched_*), the rest through the plain FP64
    form one property at a time, in file order within each list."""
    batches: list          # list of lists of property names
    plain: list            # property names


def _batchable(opt: PropertyOptions) -> bool:
    """The options the batched form takes (mohid_ad_batched_create's list in
    include/mohid_ad.h): explicit UpwindOrder1 or P2_TVD horizontal advection,
    implicit upwind vertical advection and implicit vertical diffusion, every
    boundary condition but Orlanski, no AdvectionNudging."""
    p = opt.params
    return (not opt.implicit_h and p["AdvMethodH"] in (1, 4) and p["AdvMethodV"] == 1 and
            p["ImpExp_AdvV"] == 1.0 and p["ImpExp_DifV"] == 1.0 and p["BoundaryCondition"] != 6 and
            not p["AdvectionNudging"])


def batch_plan(data: EnterData) -> BatchPlan:
    """Group the transported properties (ADVECTION_DIFFUSION on) of a data
    file: Advection_Diffusion_Processes calls AdvectionDiffusion once per
    property with the same hydrodynamics (WP:14603-14824), so properties whose
    options (and discharge flag) are equal can share one batched step."""
    groups: dict = {}
    order: list = []
    plain: list = []
    for blk in data.blocks():
        opt = property_options(data, blk)
        if not opt.advection_diffusion:
            continue
        if not _batchable(opt):
            plain.append(opt.name)
            continue
        key = (tuple(sorted(opt.params.items())), opt.discharges)
        if key not in groups:
            groups[key] = []
            order.append(key)
        groups[key].append(opt.name)
    return BatchPlan(batches=[groups[k] for k in order], plain=plain)
