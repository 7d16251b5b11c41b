"""Oracle (test infrastructure only): the reference's .info reader restated in
Python, to check derek_info_read.

Follows Source/io.f90: io_read_param (360-830; 60-character lines at 382,
'!' anywhere skips a line, "$data" opens a block), io_freeform_read (836-882;
key before the first ':' or '=', 30 characters each), io_block_parse
(1765-1937; a block line whose first character is blank, '#' or '!' is a
comment; rows converted with the units set above the block), io_spell_check
and io_levenshtein (2545-2630; the first closest key, corrected below
distance 3), the duplicate and output_level handling (763-826), and
io_initialise's conversions (299-353) with Source/units.f90 and the CODATA
2018 constants of Source/constants.f90:70-104.
"""
import math
import os

KEYS = [  # keys_array order, Source/io.f90:1275-1325, with the parameter each sets and its kind
    ("check", "check", "l"), ("profilling", "debugging", "l"), ("n_electrons", "n_electrons", "i"),
    ("energy_tol", "energy_tol", "r"), ("xc_functional", "xc_functional", "s"),
    ("cut_off_energy", "cut_off_energy", "r"), ("g_fine_scale", "g_fine_scale", "r"),
    ("write_wvfn", "write_wvfn", "l"), ("task", "task", "s"), ("soc", "soc", "l"),
    ("max_scf", "max_scf", "i"), ("scf_method", "scf_method", "s"),
    ("electronic_temp", "electronic_temp", "r"), ("conduction_bands", "conduction_bands", "i"),
    ("write_density", "write_density", "l"), ("write_potential", "write_potential", "l"),
    ("write_state", "write_state", "l"), ("external_pot", "external_pot", "s"),
    ("kpt_mp_grid", "kpt_mp_grid", "i3"), ("write_spec", "write_spec", "l"),
    ("write_memory", "write_memory", "l"), ("print_level", "iprint", "i"),
    ("finite_barrier_height", "finite_barrier_height", "r"),
    ("finite_barrier_width", "finite_barrier_width", "r3"), ("periodic_pot_grid", "periodic_pot_grid", "i3"),
    ("periodic_pot_amp", "periodic_pot_amp", "r"), ("random_seed", "random_seed", "i"),
    ("write_formatted_potential", "write_formatted_potential", "l"), ("write_potex", "write_potex", "l"),
    ("write_formatted_density", "write_formatted_density", "l"),
    ("write_formatted_potex", "write_formatted_potex", "l"), ("output_level", "output_level", "s"),
    ("ext_efield", "ext_efield", "r3"), ("ext_bfield", "ext_bfield", "r3"),
    ("unit_energy", "unit_energy", "s"), ("unit_length", "unit_length", "s"),
    ("unit_efield", "unit_efield", "s"), ("unit_bfield", "unit_bfield", "s"),
    ("unit_energy_out", "out_energy_unit", "s"), ("unit_length_out", "out_len_unit", "s"),
    ("unit_efield_out", "out_efield_unit", "s"), ("unit_bfield_out", "out_bfield_unit", "s"),
    ("lattice", None, None), ("dos_kpt_mp_grid", "dos_kpt_mp_grid", "i3"), ("write_xsf", "write_xsf", "l"),
]


def units():
    """Value of each unit in atomic units (Source/units.f90:36-127)."""
    c, h, e, me, na, r = 299792458.0, 6.62607015e-34, 1.602176634e-19, 9.1093837015e-31, 6.02214076e23, 8.314462618
    pi = math.pi
    twopi = 2.0 * pi
    hbar = h / twopi
    mu0 = 4.0 * pi * 1.0e-7
    eps0 = 1.0 / (mu0 * (c * c))
    alpha = (e * e) / (4.0 * pi * eps0 * hbar * c)
    kb = r / na
    metre = me * c * alpha / hbar
    joule = 1.0 / ((alpha * alpha) * me * (c * c))
    ev = e / ((alpha * alpha) * me * (c * c))
    inv = 1.0 / metre
    ang = metre * 1e-10
    hz = h * joule
    return {"bohr": 1.0, "m": metre, "cm": metre * 1e-2, "mm": metre * 1e-3, "mum": metre * 1e-6,
            "nm": metre * 1e-9, "A": ang, "pm": metre * 1e-12, "Ha": 1.0, "mHa": 1e-3, "eV": ev,
            "meV": ev * 1e-3, "Ry": 0.5, "mRy": 0.5 * 1e-3, "J": joule, "Hz": hz, "MHz": hz * 1e6,
            "GHz": hz * 1e9, "THz": hz * 1e12, "cm-1": hz * c * 1e2, "K": kb * joule,
            "T": e * (inv * inv) * twopi / h, "G": 1.0e-4 * e * (inv * inv) * twopi / h, "agr": 1.0,
            "Ha/Bohr/e": 1.0, "eV/A/e": ev / ang, "N/C": joule / (metre / e)}


class InfoError(Exception):
    pass


def defaults():
    p = dict(check=0, debugging=0, n_electrons=1, energy_tol=1.0e-7, xc_functional="lda",
             cut_off_energy=200.0, g_fine_scale=2.0, write_wvfn=0, task="singlepoint", soc=0, max_scf=40,
             scf_method="EDFT", electronic_temp=0.0, conduction_bands=20, write_density=0,
             write_potential=0, write_state=1, external_pot="jelly", kpt_mp_grid=[1, 1, 1], write_spec=1,
             write_memory=0, iprint=1, finite_barrier_height=10.0, finite_barrier_width=[0.5, 0.5, 0.5],
             periodic_pot_grid=[1, 1, 1], periodic_pot_amp=10.0, random_seed=0, write_formatted_potential=0,
             write_potex=0, write_formatted_density=0, restart=0, write_formatted_potex=0,
             output_level="minimal", ext_efield=[0.0] * 3, ext_bfield=[0.0] * 3, unit_energy="eV",
             unit_length="A", unit_efield="eV/A/e", unit_bfield="T", out_energy_unit="eV", out_len_unit="A",
             out_efield_unit="eV/A/e", out_bfield_unit="G", dos_kpt_mp_grid=[11, 11, 11], write_xsf=0,
             cell=[0.0] * 9, n_pots=0, pot_centres=[], pot_heights=[], pot_widths=[], n_corrected=0)
    p["xc_functional"] = "LDA"
    return p


def lev(a, b):
    d = [[0] * (len(b) + 1) for _ in range(len(a) + 1)]
    for i in range(len(a) + 1):
        d[i][0] = i
    for j in range(len(b) + 1):
        d[0][j] = j
    for i in range(1, len(a) + 1):
        for j in range(1, len(b) + 1):
            d[i][j] = min(d[i - 1][j] + 1, d[i][j - 1] + 1, d[i - 1][j - 1] + (a[i - 1] != b[j - 1]))
    return d[len(a)][len(b)]


def list_items(s, with_slash=False):
    """Values of a list-directed record: blank/comma separated, quotes,
    r*c repeats, '/' ends (with_slash: also report whether one did)."""
    out, i, slash = [], 0, False
    while i < len(s):
        while i < len(s) and s[i] in " ,":
            i += 1
        if i < len(s) and s[i] == "/":
            slash = True
            break
        if i >= len(s):
            break
        if s[i] in "'\"":
            q, i, tok = s[i], i + 1, ""
            while i < len(s):
                if s[i] == q:
                    if i + 1 < len(s) and s[i + 1] == q:
                        tok += q
                        i += 2
                        continue
                    i += 1
                    break
                tok += s[i]
                i += 1
            out.append(tok)
            continue
        j = i
        while j < len(s) and s[j] not in " ,/":
            j += 1
        tok = s[i:j]
        i = j
        star = tok.find("*")
        if star > 0 and tok[:star].isdigit():
            out += [tok[star + 1:]] * int(tok[:star])
        else:
            out.append(tok)
    return (out, slash) if with_slash else out


def real(t):
    import re
    m = re.fullmatch(r"([+-]?(?:\d+\.?\d*|\.\d+))(?:[eEdDqQ]([+-]?\d+)|([+-]\d+))?", t)
    if not m:
        raise InfoError("bad real")
    ex = m.group(2) if m.group(2) is not None else m.group(3)
    return float(m.group(1) + ("e" + ex if ex is not None else ""))


def integer(t):
    import re
    if not re.fullmatch(r"[+-]?\d+", t):
        raise InfoError("bad integer")
    return int(t)


def logical(t):
    t = t[1:] if t.startswith(".") else t
    if not t or t[0].lower() not in "tf":
        raise InfoError("bad logical")
    return 1 if t[0].lower() == "t" else 0


def read_info(path):
    u = units()

    def to_atomic(x, unit):
        if unit not in u:
            raise InfoError("Unknown unit: " + unit)
        return x * u[unit]

    p = defaults()
    with open(path) as f:
        lines = [l.rstrip("\n").rstrip("\r") for l in f]
    present, cell_declared, notes, i = [], False, [], 0
    while i < len(lines):
        line = lines[i][:60].rstrip(" ")
        i += 1
        if line == "" or "!" in line:
            continue
        if "$data" in line.lower():
            before = p["external_pot"]
            hdr = list_items(line.lower().strip(" "))
            tin = hdr[1][:20]
            j = i
            while True:
                if j >= len(lines):
                    raise InfoError("Block not closed")
                b = lines[j][:300].lower().strip(" ")
                if "$enddata" in b:
                    if list_items(b)[1][:20] != tin:
                        raise InfoError("Block not closed")
                    break
                j += 1
            data = [l[:300] for l in lines[i:j] if not (l[:1] in ("", " ", "#", "!"))]
            if not data:
                raise InfoError("No data in block")
            if tin == "lattice":
                if len(data) != 3:
                    raise InfoError("LATTICE must have 3 lines")
                for r, row in enumerate(data):
                    v = [real(x) for x in list_items(row)[:3]]
                    for c in range(3):
                        p["cell"][r + 3 * c] = to_atomic(v[c], p["unit_length"])
                cell_declared = True
            elif tin in ("gaussian_pot", "lorentzian_pot"):
                p["external_pot"] = tin
                p["n_pots"] = len(data)
                for row in data:
                    v = [real(x) for x in list_items(row)[:5]]
                    p["pot_centres"] += v[:3]
                    p["pot_heights"].append(to_atomic(v[3], p["unit_energy"]))
                    p["pot_widths"].append(to_atomic(v[4], p["unit_length"]))
            else:
                raise InfoError("Unknown block type")
            if p["external_pot"] != before:
                present.append("external_pot")
            i = j + 1
            continue
        if line[0] in "!#":
            continue
        seps = [k for k in (line.find(":"), line.find("=")) if k >= 0]
        if not seps:
            raise InfoError("Error parsing line")
        sep = min(seps)
        key = line[:sep][:30].lower().strip(" ")
        val = line[sep + 1:][:30]
        if "unit" not in key:
            val = val.lower().strip(" ")
        dists = [lev(key, k[0]) for k in KEYS]
        best = min(dists)
        if best >= 3:
            raise InfoError("Unknown parameter - " + key)
        name, field, kind = KEYS[dists.index(best)]
        if best > 0:
            notes.append(f"{key} -> {name}")
            p["n_corrected"] += 1
        if field is None:
            raise InfoError("Error parsing keyword")
        items, slash = list_items(val, with_slash=True)
        need = 3 if kind in ("i3", "r3") else 1
        if len(items) < need and not slash:
            raise InfoError("Error parsing value")
        conv = {"l": logical, "i": integer, "r": real, "s": lambda x: x[:30], "i3": integer, "r3": real}[kind]
        if need == 1:
            if items:
                p[field] = conv(items[0])
        else:   # a '/' leaves the remaining elements as they were
            p[field] = [conv(items[c]) if c < len(items) else p[field][c] for c in range(3)]
        if name == "task" and p["task"] not in ("singlepoint", "bandstructure", "dos"):
            raise InfoError("Unknown task")
        if name == "external_pot":
            e = p["external_pot"]
            if e in ("gaussian_pot", "lorentzian_pot"):
                raise InfoError("block only")
            if e not in ("jelly", "finite_barrier", "periodic_pot"):
                if not os.path.exists(e):
                    raise InfoError("Potential file does not exist")
                if "potex" not in e:
                    raise InfoError("Unsupported external potential file")
        if name == "print_level" and not 1 <= p["iprint"] <= 3:
            raise InfoError("print_level")
        present.append(name)
    if len(set(present)) != len(present):
        raise InfoError("Duplicate parameter")
    if "output_level" in present:
        flags = ["write_wvfn", "write_spec", "write_state", "write_potex", "write_formatted_potex",
                 "write_density", "write_formatted_density", "write_potential", "write_formatted_potential"]
        vals = {"minimal": [0, 0, 1, 1, 0, 1, 0, 0, 0], "none": [0] * 9, "all": [1] * 9}.get(p["output_level"])
        if vals:
            for f, v in zip(flags, vals):
                p[f] = v
    if p["task"] in ("bandstructure", "dos"):
        p["write_spec"] = 1
    if not cell_declared:
        raise InfoError("No lattice provided")
    p["nbands"] = p["n_electrons"] + p["conduction_bands"]
    for f in ("energy_tol", "cut_off_energy", "finite_barrier_height", "periodic_pot_amp"):
        p[f] = to_atomic(p[f], p["unit_energy"])
    p["electronic_temp"] = to_atomic(p["electronic_temp"], "K")
    p["finite_barrier_width"] = [to_atomic(x, p["unit_length"]) for x in p["finite_barrier_width"]]
    p["ext_efield"] = [to_atomic(x, p["unit_efield"]) for x in p["ext_efield"]]
    p["ext_bfield"] = [to_atomic(x, p["unit_bfield"]) for x in p["ext_bfield"]]
    p["corrected"] = notes
    return p
