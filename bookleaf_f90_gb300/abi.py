"""ctypes mirror of include/bookleaf_gb300.h.

The structs below must match the C header field for field; tests check the
sizes against the compiled library (``bl_abi_sizes``).
"""
import ctypes as ct

NID = 79
MAXMAT = 100
MAXREG = 100
NEOSPARAM = 6
SLEN = 130

# dataAPI field IDs (src/dataAPI/dataAPI_id.f90:26-74)
IDS = dict(
    ELDENSITY=1, ELENERGY=2, ELPRESSURE=3, ELCS2=4, ELVOLUME=5, A1=6, A2=7, A3=8,
    B1=9, B2=10, B3=11, CNWT=12, CNX=13, CNY=14, RSCRATCH21=15, RSCRATCH22=16,
    RSCRATCH23=17, RSCRATCH24=18, RSCRATCH25=19, RSCRATCH26=20, RSCRATCH27=21,
    RSCRATCH28=22, CNVISCX=23, CNVISCY=24, ELVISC=25, ELMASS=26, CNMASS=27,
    RSCRATCH11=28, RSCRATCH12=29, RSCRATCH13=30, RSCRATCH14=31, RSCRATCH15=32,
    RSCRATCH16=33, RSCRATCH17=34, NDX=35, NDY=36, NDU=37, NDV=38, INDTYPE=39,
    IELSORT1=40, IELND=41, IELEL=42, IELFC=43, IELMAT=44, IELREG=45, IELSORT2=46,
    SPMASS=47, ISCRATCH11=48, ZSCRATCH11=49, IELLOCGLOB=50, INDLOCGLOB=51,
    CPDENSITY=52, CPENERGY=53, CPPRESSURE=54, CPCS2=55, CPVOLUME=56, FRVOLUME=57,
    CPMASS=58, FRMASS=59, CPVISCX=60, CPVISCY=61, CPVISC=62, CPA1=63, CPA3=64,
    CPB1=65, CPB3=66, ICPMAT=67, ICPNEXT=68, ICPPREV=69, IMXEL=70, IMXFCP=71,
    IMXNCP=72, ICPSCRATCH11=73, ICPSCRATCH12=74, RCPSCRATCH11=75,
    RCPSCRATCH21=76, RCPSCRATCH22=77, RCPSCRATCH23=78, RCPSCRATCH24=79,
)
globals().update(IDS)
NAMES = {v: k.lower() for k, v in IDS.items()}

SUCCESS, FAILURE, HALT_ALL, HALT_SINGLE = 0, -1, 1, 2
FP_FAST, FP_EXACT, FP_MIXED = 0, 1, 2
DT_NAMES = [" MAXIMUM", "  GROWTH", " INITIAL", "     CFL", "     DIV"]


class Sizes(ct.Structure):
    """sizes_t (src/dataAPI/dataAPI_types.f90:40-43)."""
    _fields_ = [(n, ct.c_int) for n in (
        "nel", "nel1", "nel2", "nnd", "nnd1", "nnd2", "nsz", "nmat", "nreg",
        "ncp", "nmx", "mcp", "mmx")]


class Config(ct.Structure):
    """Flattened config_t subset read by the hot path."""
    _fields_ = [
        ("time_start", ct.c_double), ("time_end", ct.c_double),
        ("dt_g", ct.c_double), ("dt_min", ct.c_double),
        ("dt_max", ct.c_double), ("dt_initial", ct.c_double),
        ("cvisc1", ct.c_double), ("cvisc2", ct.c_double),
        ("cfl_sf", ct.c_double), ("div_sf", ct.c_double),
        ("ztq", ct.c_int), ("zhg", ct.c_int), ("zsp", ct.c_int), ("pad0", ct.c_int),
        ("kappareg", ct.c_double * MAXREG), ("pmeritreg", ct.c_double * MAXREG),
        ("zdtnotreg", ct.c_int * MAXREG), ("zmidlength", ct.c_int * MAXREG),
        ("zcut", ct.c_double), ("zerocut", ct.c_double),
        ("dencut", ct.c_double), ("accut", ct.c_double),
        ("ccut", ct.c_double), ("pcut", ct.c_double),
        ("eos_type", ct.c_int * (MAXMAT + 1)), ("pad1", ct.c_int),
        ("eos_param", (ct.c_double * NEOSPARAM) * (MAXMAT + 1)),
        ("ale_zexist", ct.c_int), ("ale_zon", ct.c_int), ("ale_zeul", ct.c_int),
        ("ale_adv_type", ct.c_int), ("ale_npatch", ct.c_int), ("pad2", ct.c_int),
        ("ale_mintime", ct.c_double), ("ale_maxtime", ct.c_double),
        ("ale_sf", ct.c_double),
    ]


class Timestep(ct.Structure):
    """timestep_t (src/dataAPI/dataAPI_types.f90:45-51)."""
    _fields_ = [
        ("time", ct.c_double), ("dt", ct.c_double), ("dts", ct.c_double),
        ("nstep", ct.c_int), ("idtel", ct.c_int), ("zcorrector", ct.c_int),
        ("imdt", ct.c_int), ("sdt", ct.c_char * 9), ("mdt", ct.c_char * 11),
    ]

    def copy(self):
        t = Timestep()
        ct.pointer(t)[0] = self
        return t

    def as_tuple(self):
        return (self.nstep, self.time, self.dt, self.dts, self.idtel,
                self.zcorrector, self.sdt, self.imdt)


class Error(ct.Structure):
    """error_t (src/dataAPI/dataAPI_types.f90:76-79)."""
    _fields_ = [("ierr", ct.c_int), ("iout", ct.c_int), ("serr", ct.c_char * (SLEN + 1))]

    @property
    def message(self):
        return self.serr.decode(errors="replace").strip()


class StepRecord(ct.Structure):
    _fields_ = [("time", ct.c_double), ("dt", ct.c_double), ("nstep", ct.c_int),
                ("idtel", ct.c_int), ("sdt_code", ct.c_int), ("ierr", ct.c_int)]


def pointer_table(arrays):
    """Host pointer table indexed by dataAPI ID (entry 0 unused)."""
    tab = (ct.c_void_p * (NID + 1))()
    for fid, arr in arrays.items():
        if arr is not None:
            tab[fid] = arr.ctypes.data
    return tab
