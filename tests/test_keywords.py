"""MOHID keyword data files (ModuleEnterData) and the advection-diffusion
options of a WaterProperties file (Read_Advec_Difus_Parameters,
ModuleWaterProperties.F90:9226-9733)."""
import numpy as np
import pytest

from mohid_gb300 import keywords as K

FILE = """\
! a WaterProperties data file
OUTPUT_TIME              : 0  3600
ADV_METHOD_H            : 4          ! P2_TVD, read for every property
\tTVD_LIMIT_H           : 1
VOLUME_RELATION_MAX     : 2.5d0
FILENAME                : C:\\data\\run\\file.hdf5

<beginproperty>
NAME                         : salinity
ADVECTION_DIFFUSION          : 1
BOUNDARY_CONDITION           : 4
DISCHARGES                   : 1
SCHMIDT_BACKGROUND_V         : 1.e-6
DIFFUSION_V_IMP_EXP          : 0.5
<endproperty>

<beginproperty>
NAME                         : temperature
ADVECTION_DIFFUSION          :
ADVECTION_H_IMP_EXP          : 0
ADV_METHOD_H                 : 1          ! inside a block: not the file's method
<endproperty>

<beginproperty>
NAME                         : cohesive sediment
ADVECTION_DIFFUSION          : 0
ADVECTION_NUDGING            : 1
<endproperty>
"""


def test_enter_data_syntax():
    d = K.EnterData(FILE)
    assert d.integer("ADV_METHOD_H", 0) == 4            # comment stripped, first match
    assert d.integer("TVD_LIMIT_H", 0) == 1             # tab and leading blanks
    assert d.real("VOLUME_RELATION_MAX", 0.0) == 2.5    # Fortran d exponent
    assert d.real("OUTPUT_TIME", -1.0) == 0.0           # first value of a list
    assert d.string("FILENAME") == "C:\\data\\run\\file.hdf5"
    assert d.real("ABSENT", 7.0) == 7.0
    blocks = d.blocks()
    assert len(blocks) == 3
    assert d.string("NAME", block=blocks[1]) == "temperature"
    assert d.integer("ADV_METHOD_H", 0, block=blocks[1]) == 1
    assert d.integer("ADV_METHOD_H", 0, block=blocks[0]) == 0   # not in the first block
    # a logical with nothing readable counts as 1
    assert d.logical("ADVECTION_DIFFUSION", False, block=blocks[1]) is True
    assert d.logical("ADVECTION_DIFFUSION", True, block=blocks[2]) is False


def test_enter_data_errors():
    with pytest.raises(K.KeywordError):
        K.EnterData("NULLDIF 1\n").logical("NULLDIF", False)          # no ':' delimiter
    with pytest.raises(K.KeywordError):
        K.EnterData("NULLDIF : 2\n").logical("NULLDIF", False)        # logical not 0 or 1
    with pytest.raises(K.KeywordError):
        K.EnterData("DECAY_TIME : soon\n").real("DECAY_TIME", 0.0)
    with pytest.raises(K.KeywordError):
        K.EnterData("<beginproperty>\nNAME : a\n").blocks()            # unterminated block
    # case sensitive, as ModuleEnterData by default
    assert K.EnterData("nulldif : 1\n").logical("NULLDIF", False) is False


def test_property_options():
    d = K.EnterData(FILE)
    sal, tem, sed = (K.property_options(d, b) for b in d.blocks())
    assert (sal.name, sal.advection_diffusion, sal.discharges, sal.implicit_h) == ("salinity", True, True, False)
    p = sal.params
    # methods and limiters from the file, the rest from the block or the defaults
    assert (p["AdvMethodH"], p["TVDLimitationH"], p["Upwind2H"]) == (4, 1, 1)
    assert (p["AdvMethodV"], p["TVDLimitationV"], p["Upwind2V"]) == (1, 4, 0)
    assert p["VolumeRelMax"] == 2.5
    assert p["BoundaryCondition"] == 4 and p["SchmidtBackground_V"] == 1e-6
    assert p["ImpExp_DifV"] == 0.5 and p["ImpExp_AdvV"] == 1.0
    assert tem.implicit_h and tem.params["AdvMethodH"] == 4                  # the file's method
    assert K.step_directions(tem, 0) == dict(ImpExp_AdvXX=1.0, ImpExp_AdvYY=0.0)
    assert K.step_directions(tem, 1) == dict(ImpExp_AdvXX=0.0, ImpExp_AdvYY=1.0)
    assert K.step_directions(sal, 3) == dict(ImpExp_AdvXX=0.0, ImpExp_AdvYY=0.0)
    assert not sed.advection_diffusion
    assert sed.params["AdvectionNudging"] == 1 and sed.params["AdvectionNudgingCells"] == 10


def test_defaults_equal_the_library_defaults():
    # an empty property block gives the reference's defaults, which
    # mohid_ad_default_params also holds
    from mohid_gb300 import advdiff
    d = K.EnterData("<beginproperty>\nNAME : x\n<endproperty>\n")
    opt = K.property_options(d, d.blocks()[0])
    lib = advdiff.params()
    for k, v in opt.params.items():
        assert getattr(lib, k) == v, k


def test_rejected_options():
    with pytest.raises(K.KeywordError):                  # ERR100: no such boundary condition
        d = K.EnterData("<beginproperty>\nBOUNDARY_CONDITION : 3\n<endproperty>\n")
        K.property_options(d, d.blocks()[0])
    with pytest.raises(K.KeywordError):                  # ERR190: implicit H with UpwindOrder2
        d = K.EnterData("ADV_METHOD_H : 2\n<beginproperty>\nADVECTION_H_IMP_EXP : 0\n<endproperty>\n")
        K.property_options(d, d.blocks()[0])


def test_options_drive_the_oracle(built):
    # the options read from a file are a valid argument set: the oracle steps with them
    from oracle import oracle as O
    from tests.cases import domain
    dom = domain("open")
    d = K.EnterData(FILE)
    for b in d.blocks()[:2]:
        opt = K.property_options(d, b)
        p = dict(opt.params, DTProp=30.0, **K.step_directions(opt, 0))
        P = dom.tracer(3, 1.0, 0.5, seed=1)
        R = dom.reference(2.0, 0.3, seed=2)
        assert O.step(dom, P, O.params(**p), ReferenceProp=R) == 0
        assert np.isfinite(P).all()


def test_batch_plan():
    text = """ADV_METHOD_H : 4
TVD_LIMIT_H : 4
<beginproperty>
NAME : temperature
<endproperty>
<beginproperty>
NAME : salinity
<endproperty>
<beginproperty>
NAME : fecal coliforms
DECAY_TIME : 86400.
<endproperty>
<beginproperty>
NAME : oxygen
DISCHARGES : 1
<endproperty>
<beginproperty>
NAME : nitrate
DISCHARGES : 1
<endproperty>
<beginproperty>
NAME : ammonia
ADVECTION_H_IMP_EXP : 0
<endproperty>
<beginproperty>
NAME : sediment
BOUNDARY_CONDITION : 6
<endproperty>
<beginproperty>
NAME : chlorophyll
ADVECTION_NUDGING : 1
<endproperty>
<beginproperty>
NAME : age
ADVECTION_DIFFUSION : 0
<endproperty>
"""
    plan = K.batch_plan(K.EnterData(text))
    # equal options share a batch; decay time and discharges make their own;
    # implicit horizontal advection, Orlanski and nudging go to the plain form;
    # untransported properties appear nowhere
    assert plan.batches == [["temperature", "salinity"], ["fecal coliforms"], ["oxygen", "nitrate"]]
    assert plan.plain == ["ammonia", "sediment", "chlorophyll"]
