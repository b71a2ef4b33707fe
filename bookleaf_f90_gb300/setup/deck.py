"""Control-file reader for the reference's namelist decks.

Reads the subset of BookLeaf's control-file namelists that the hot path
needs -- CONTROL, EOS, CUTOFF, ALE, MESH, INDICATORS, SHAPES and
INITIAL_CONDITIONS -- with the reference's defaults and rationalisation:

  CONTROL              setup_read.f90:113-253 (defaults time_config.f90,
                       hydro_config.f90:32-82; rationalise hydro_config.f90:292-414)
  ALE                  setup_read.f90:255-431, ale_config.f90:31-117, 511-551
  CUTOFF               setup_read.f90:467-507, global_config.f90:32-42,
                       eos_config.f90:31-60
  EOS                  setup_read.f90:509-589, eos_config.f90:163-226
  MESH                 setup_mesh.F90:106-346
  INDICATORS           setup_IC.f90:813-1122
  SHAPES               setup_IC.f90:1124-1208
  INITIAL_CONDITIONS   setup_IC.f90:1210-1419

Only Fortran namelist syntax the reference decks use is accepted:
``name = v``, ``name(i) = v``, ``name(i,j) = v``, array sections with ``:``
or ``a:b`` filled in column-major order by a value list, strings in quotes,
logicals ``.TRUE.``/``.FALSE.``.  Unknown groups are ignored.
"""
import re

import numpy as np

from .. import abi

LN = 100          # setup_read.f90:31, setup_IC.f90:82
LI = 100          # setup_mesh.F90:115
HUGE = np.finfo(np.float64).max


class DeckError(ValueError):
    """A control file the reference would reject (same messages)."""


_group_re = re.compile(r"&(\w+)(.*?)(?:^\s*/\s*$|\n\s*/)", re.S | re.M)


def _strip_comments(text):
    out = []
    for line in text.splitlines():
        q = None
        cut = len(line)
        for i, ch in enumerate(line):
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch == "!":
                cut = i
                break
        out.append(line[:cut])
    return "\n".join(out)


def _tokens(body):
    """Split a namelist group body into (key, [raw values]) pairs."""
    toks = []
    i, n = 0, len(body)
    cur = ""
    items = []
    while i < n:
        ch = body[i]
        if ch in "'\"":
            j = body.index(ch, i + 1)
            items.append(("S", body[i + 1:j]))
            i = j + 1
            continue
        if ch == "(":
            j = body.index(")", i)
            cur += body[i:j + 1]
            i = j + 1
            continue
        if ch in ",\n\t ":
            if cur.strip():
                items.append(("W", cur.strip()))
            cur = ""
            i += 1
            continue
        if ch == "=":
            if cur.strip():
                items.append(("W", cur.strip()))
            cur = ""
            items.append(("=", "="))
            i += 1
            continue
        cur += ch
        i += 1
    if cur.strip():
        items.append(("W", cur.strip()))
    # assemble key = values
    k = 0
    while k < len(items):
        if k + 1 < len(items) and items[k + 1][0] == "=":
            key = items[k][1]
            k += 2
            vals = []
            while k < len(items) and not (k + 1 < len(items) and items[k + 1][0] == "="):
                vals.append(items[k])
                k += 1
            toks.append((key, vals))
        else:
            raise DeckError("ERROR: namelist syntax near %r" % (items[k][1],))
    return toks


def _value(tok):
    kind, s = tok
    if kind == "S":
        return s
    u = s.upper()
    if u in (".TRUE.", "T", ".T.", "TRUE"):
        return True
    if u in (".FALSE.", "F", ".F.", "FALSE"):
        return False
    try:
        if re.fullmatch(r"[+-]?\d+", s):
            return int(s)
        return float(s.replace("d", "e").replace("D", "e"))
    except ValueError:
        return s


def _indices(sub, ndim_ext):
    """Index tuples (1-based) of an array section, column-major order."""
    parts = [p.strip() for p in sub.split(",")]
    ranges = []
    for d, p in enumerate(parts):
        ext = ndim_ext[d] if d < len(ndim_ext) else LN
        if p == ":":
            ranges.append(list(range(1, ext + 1)))
        elif ":" in p:
            a, b = p.split(":")
            a = int(a) if a.strip() else 1
            b = int(b) if b.strip() else ext
            ranges.append(list(range(a, b + 1)))
        else:
            ranges.append([int(p)])
    # column-major: the first dimension varies fastest
    idx = [[]]
    for r in ranges:
        idx = [prev + [v] for v in r for prev in idx]
    return [tuple(t) for t in idx]


class Namelist(dict):
    """One group: name -> scalar, or name -> {index tuple: value}."""

    def get_scalar(self, name, default):
        v = self.get(name.lower(), None)
        if v is None:
            return default
        if isinstance(v, dict):
            return v.get((1,), default)
        return v

    def get_array(self, name, shape, default):
        arr = np.empty(shape, dtype=object)
        arr[...] = default
        v = self.get(name.lower(), None)
        if v is None:
            return arr
        if not isinstance(v, dict):
            v = {(1,) * len(shape): v}
        for idx, val in v.items():
            if len(idx) < len(shape):
                idx = idx + (1,) * (len(shape) - len(idx))
            arr[tuple(i - 1 for i in idx)] = val
        return arr


_EXTENTS = {
    "region_side": (LI, 4, LI), "region_dim": (LI, 2), "segment_pos": (LI, 8),
    "eos_param": (6, LN), "kinematic_param": (3, LN), "shape_param": (LN, 5),
    "patch_trigger": (LN, LN),
}


def parse(text):
    """Parse every namelist group of a control file."""
    text = _strip_comments(text)
    groups = {}
    for m in re.finditer(r"&(\w+)", text):
        name = m.group(1).lower()
        start = m.end()
        # the group ends at the first '/' outside quotes
        q = None
        j = start
        while j < len(text):
            ch = text[j]
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch == "/":
                break
            j += 1
        body = text[start:j]
        nl = Namelist()
        for key, vals in _tokens(body):
            km = re.fullmatch(r"(\w+)\s*(?:\((.*)\))?", key)
            if not km:
                raise DeckError("ERROR: bad namelist item %r" % key)
            var, sub = km.group(1).lower(), km.group(2)
            values = [_value(v) for v in vals]
            if sub is None and len(values) == 1:
                nl[var] = values[0]
                continue
            if sub is None:
                sub = ":"
            ext = _EXTENTS.get(var, (LN,) * (sub.count(",") + 1))
            idx = _indices(sub, ext)
            if len(values) > len(idx):
                raise DeckError("ERROR: too many values for %s" % var)
            d = nl.setdefault(var, {})
            if not isinstance(d, dict):
                d = {(1,): d}
                nl[var] = d
            for t, v in zip(idx, values):
                d[t] = v
        groups[name] = nl
    return groups


def read_deck(path_or_text):
    """Return the parsed groups of a control file (path or text)."""
    if "\n" in path_or_text or "&" in path_or_text:
        text = path_or_text
    else:
        with open(path_or_text) as f:
            text = f.read()
    return parse(text)


def build_config(groups, nreg, nmat):
    """config_t after the reference's defaults, namelists and rationalise.

    nreg/nmat come from the INDICATORS group (setup_indicator_types)."""
    c = abi.Config()
    ctl = groups.get("control", Namelist())
    # time_cf_defaults (time_config.f90)
    c.time_start = float(ctl.get_scalar("time_start", 0.0))
    c.time_end = float(ctl.get_scalar("time_end", 1.0))
    c.dt_initial = float(ctl.get_scalar("dt_initial", 1.0e-5))
    c.dt_g = float(ctl.get_scalar("dt_g", 1.02))
    c.dt_min = float(ctl.get_scalar("dt_min", 1.0e-8))
    c.dt_max = float(ctl.get_scalar("dt_max", 1.0e-1))
    if c.time_start > c.time_end:
        raise DeckError("ERROR: time_start > time_end")
    if c.dt_min > c.dt_max:
        raise DeckError("ERROR: dt_min > dt_max")
    # hydro_cf_defaults (hydro_config.f90:42-77)
    c.cvisc1 = float(ctl.get_scalar("cvisc1", 0.5))
    c.cvisc2 = float(ctl.get_scalar("cvisc2", 0.75))
    c.cfl_sf = float(ctl.get_scalar("cfl_sf", 0.5))
    c.div_sf = float(ctl.get_scalar("div_sf", 0.25))
    visc = str(ctl.get_scalar("visc", "EDGE")).upper()
    if visc not in ("EDGE", "TENSOR"):
        raise DeckError("ERROR: unknown value of visc")
    c.ztq = int(visc == "TENSOR")
    for nm in ("cvisc1", "cvisc2", "cfl_sf", "div_sf"):
        if getattr(c, nm) < 0.0:
            raise DeckError("ERROR: %s < 0" % nm)
    kappaall = float(ctl.get_scalar("kappaall", 0.0))
    pmeritall = float(ctl.get_scalar("pmeritall", 0.0))
    kreg = ctl.get_array("kappareg", (LN,), 0.0)
    preg = ctl.get_array("pmeritreg", (LN,), 0.0)
    zdt = ctl.get_array("zdtnotreg", (LN,), False)
    zml = ctl.get_array("zmidlength", (LN,), False)
    # setup_read.f90:239,250: MERGE(kappareg,kappaall,kappareg>0)
    for i in range(nreg):
        k = float(kreg[i])
        c.kappareg[i] = k if k > 0.0 else kappaall
        p = float(preg[i])
        c.pmeritreg[i] = p if p > 0.0 else pmeritall
        c.zdtnotreg[i] = int(bool(zdt[i]))
        c.zmidlength[i] = int(bool(zml[i]))
    # hydro_cf_rationalise (hydro_config.f90:349,368)
    c.zhg = int(any(c.kappareg[i] > 0.0 for i in range(nreg)))
    c.zsp = int(any(c.pmeritreg[i] > 0.0 for i in range(nreg)))
    # global_cf_defaults / eos_cf_defaults, then CUTOFF
    cut = groups.get("cutoff", Namelist())
    c.zcut = float(cut.get_scalar("zcut", 1.0e-8))
    c.zerocut = float(cut.get_scalar("zerocut", 1.0e-40))
    c.dencut = float(cut.get_scalar("dencut", 1.0e-6))
    c.accut = float(cut.get_scalar("accut", 1.0e-6))
    c.ccut = float(cut.get_scalar("ccut", 1.0e-6))
    c.pcut = float(cut.get_scalar("pcut", 1.0e-8))
    for nm in ("zcut", "zerocut", "dencut", "accut", "ccut", "pcut"):
        if getattr(c, nm) < 0.0:
            raise DeckError("ERROR: %s < 0" % nm)
    # EOS (setup_read.f90:509-589; eos_config.f90:163-226)
    eos = groups.get("eos", Namelist())
    etype = eos.get_array("eos_type", (LN,), "UNKNOWN")
    # eos_cf_defaults holds param(2,1)=-1, replicated over LN by eos_cf_get
    # (eos_config.f90:55-58, 94-107); rows 3..6 start at zero here.
    eparam = eos.get_array("eos_param", (6, LN), None)
    for m in range(LN):
        for k in range(6):
            if eparam[k, m] is None:
                eparam[k, m] = -1.0 if k < 2 else 0.0
    names = {"UNKNOWN": -1, "VOID": 0, "IDEAL GAS": 1, "TAIT": 2, "JWL": 3}
    c.eos_type[0] = 0
    for k in range(6):
        c.eos_param[0][k] = 0.0
    for m in range(1, nmat + 1):
        t = str(etype[m - 1]).upper().strip()
        if t not in names:
            raise DeckError("ERROR: unrecognised EoS type")
        c.eos_type[m] = names[t]
        for k in range(6):
            v = eparam[k, m - 1]
            # eos_cf_defaults sizes param (2,1) with -1; unset entries read 0
            c.eos_param[m][k] = float(v) if v is not None else 0.0
    # ALE (ale_config.f90:42-49, 511-551)
    ale = groups.get("ale", Namelist())
    c.ale_adv_type = int(ale.get_scalar("adv_type", 1))
    c.ale_npatch = int(ale.get_scalar("npatch", 0))
    c.ale_sf = float(ale.get_scalar("ale_sf", 0.5))
    c.ale_zeul = int(bool(ale.get_scalar("zeul", False)))
    c.ale_zon = 0                      # no input sets ale%zon
    c.ale_mintime = HUGE
    c.ale_maxtime = HUGE
    c.ale_zexist = 0
    if c.ale_zeul:
        c.ale_npatch = 1
        c.ale_mintime = -HUGE
        c.ale_maxtime = HUGE
        c.ale_zexist = 1
    elif c.ale_npatch < 0:
        raise DeckError("ERROR: npatch < 0")
    return c
