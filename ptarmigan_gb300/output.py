"""Distribution output: the reference's DistributionFunction (output/mod.rs:
173-343) over histograms generated on the device (ptg_histogram), with its
unit systems (output/units.rs) and its plain-text file format
(output/hgram.rs:530-562).

    dstr = DistributionFunction.load("energy:(log;energy)")
    dstr.write(engine, particles, abi.PHOTON, UnitSystem.default(), "out/photon")

Filter bounds are numbers or "auto" (the reference's own expression
evaluator is not part of this package).
"""

import math

import numpy as np

from . import abi

# constants.rs
ELEMENTARY_CHARGE = 1.602177e-19
SPEED_OF_LIGHT = 2.997925e8

# output/functions.rs:10-105: name -> (device function, output type)
_DIMLESS, _ANGLE, _LENGTH, _ENERGY, _MOMENTUM = range(5)
FUNCTIONS = {}
for _names, _f, _t in (
        (("angle_x",), 0, _ANGLE), (("angle_y",), 1, _ANGLE), (("theta", "pi_minus_angle"), 2, _ANGLE),
        (("angle", "polar_angle"), 3, _ANGLE), (("px", "p_x"), 4, _MOMENTUM), (("py", "p_y"), 5, _MOMENTUM),
        (("pz", "p_z"), 6, _MOMENTUM), (("p_perp",), 7, _MOMENTUM), (("r_perp",), 8, _DIMLESS),
        (("r_x", "rx"), 9, _DIMLESS), (("r_y", "ry"), 10, _DIMLESS), (("p^-", "p-", "p_minus"), 11, _MOMENTUM),
        (("p^+", "p+", "p_plus"), 12, _MOMENTUM), (("gamma",), 13, _DIMLESS), (("energy",), 14, _ENERGY),
        (("unit",), 15, _DIMLESS), (("x",), 16, _LENGTH), (("y",), 17, _LENGTH), (("z",), 18, _LENGTH),
        (("radius", "rho"), 19, _LENGTH), (("birth_a",), 20, _DIMLESS), (("parent_chi",), 21, _DIMLESS),
        (("n_inter", "n_gamma", "n_pos"), 22, _DIMLESS), (("absorption", "energy_abs"), 23, _ENERGY),
        (("weight", "number"), 29, _DIMLESS), (("S_1", "S1"), 24, _DIMLESS), (("S_2", "S2"), 25, _DIMLESS),
        (("S_3", "S3"), 26, _DIMLESS), (("pol_x", "pol_sigma"), 27, _DIMLESS), (("pol_y", "pol_pi"), 28, _DIMLESS),
        (("helicity",), 30, _DIMLESS)):
    for _n in _names:
        FUNCTIONS[_n] = (_f, _t)

# output/mod.rs:226-233
WEIGHTS = {"energy": abi.WEIGHT_ENERGY, "weight": abi.WEIGHT_NUMBER, "auto": abi.WEIGHT_NUMBER,
           "pol_x": abi.WEIGHT_POL_X, "pol_y": abi.WEIGHT_POL_Y, "helicity": abi.WEIGHT_HELICITY}


class Unit:
    """A unit: `scale` converts from the default MeV-m system."""

    def __init__(self, scale, name):
        self.scale, self.name = scale, name


class UnitSystem:
    """output/units.rs:39-80."""

    def __init__(self, length, energy, momentum):
        self.length, self.energy, self.momentum = length, energy, momentum

    @staticmethod
    def default():
        return UnitSystem(Unit(1.0, "m"), Unit(1.0, "MeV"), Unit(1.0, "MeV/c"))

    @staticmethod
    def hep():
        return UnitSystem(Unit(1.0e3, "mm"), Unit(1.0e-3, "GeV"), Unit(1.0e-3, "GeV/c"))

    @staticmethod
    def si():
        return UnitSystem(Unit(1.0, "m"), Unit(1.0e6 * ELEMENTARY_CHARGE, "J"),
                          Unit(1.0e6 * ELEMENTARY_CHARGE / SPEED_OF_LIGHT, "kg/m/s"))

    @staticmethod
    def named(s):
        """The output:units key: auto, hep or si (main.rs:925-945)."""
        table = {"auto": UnitSystem.default, "hep": UnitSystem.hep, "HEP": UnitSystem.hep, "si": UnitSystem.si,
                 "SI": UnitSystem.si}
        if s not in table:
            raise ValueError('unit system requested, "%s", is not one of "auto", "hep", or "si"' % s)
        return table[s]()

    def unit_of(self, otype):
        """ParticleOutputType::into_unit (output/mod.rs:43-53)."""
        return {_DIMLESS: Unit(1.0, "1"), _ANGLE: Unit(1.0, "rad"), _LENGTH: self.length, _ENERGY: self.energy,
                _MOMENTUM: self.momentum}[otype]


def _canonical(name):
    return {"p^-": "p_minus", "p-": "p_minus", "p^+": "p_plus", "p+": "p_plus", "rho": "radius"}.get(name, name)


def _bin_spec(s):
    """BinSpec::from (output/hgram.rs:73-88): (kind, n_bins, bin_size)."""
    try:
        n = int(s)
        if n >= 0 and str(n) == s.strip():
            return abi.BINS_FIXED_NUMBER, n, 0.0
    except ValueError:
        pass
    try:
        return abi.BINS_FIXED_SIZE, 0, float(s)
    except ValueError:
        pass
    return (abi.BINS_LOG if s == "log" else abi.BINS_AUTO), 0, 0.0


class DistributionFunction:
    """A distribution output spec such as "angle_x:angle_y:(100;energy)" or
    "energy:(log;weight;energy in 1e3, auto)"."""

    def __init__(self, names, funcs, types, bin_spec, weight, filter_):
        self.names, self.funcs, self.types = names, funcs, types
        self.dim = len(funcs)
        self.bin_spec = bin_spec
        self.weight = weight
        self.filter = filter_  # None or (name, func, min, max) in default units

    @staticmethod
    def load(spec):
        ss = spec.split(":")
        bspec, weight, filt = (abi.BINS_AUTO, 0, 0.0), "weight", None
        if len(ss) >= 2 and ss[-1].startswith("(") and ss[-1].endswith(")"):
            last = ss.pop()[1:-1].split(";")
            if len(last) == 1:
                weight = last[0].strip()
            elif len(last) == 2:
                bspec, weight = _bin_spec(last[0].strip()), last[1].strip()
            elif len(last) == 3:
                bspec, weight, filt = _bin_spec(last[0].strip()), last[1].strip(), last[2]
        if weight not in WEIGHTS or any(n not in FUNCTIONS for n in ss) or len(ss) not in (1, 2):
            raise ValueError("cannot convert %r to a distribution function" % spec)
        names = [_canonical(n) for n in ss]
        funcs = [FUNCTIONS[n][0] for n in ss]
        types = [FUNCTIONS[n][1] for n in ss]
        return DistributionFunction(names, funcs, types, bspec, weight, DistributionFunction._filter(filt, spec))

    @staticmethod
    def _filter(s, spec):
        """Filter::from_str (output/mod.rs:69-124), bounds given in SI."""
        if s is None:
            return None
        err = ValueError("cannot convert %r to a filter" % spec)
        if "," not in s:
            raise err
        prefix, suffix = s.split(",", 1)
        words = prefix.split()
        if len(words) < 3 or words[1] != "in":
            raise err
        name = _canonical(words[0])
        if name not in FUNCTIONS:
            raise err
        func, otype = FUNCTIONS[name]

        def num(t, auto):
            t = t.strip()
            if t == "auto":
                return auto
            try:
                return float(t)
            except ValueError:
                raise err
        lo = num("".join(words[2:]), -math.inf)
        hi = num(suffix, math.inf)
        # from_si multiplies by the reciprocal of the scale (output/units.rs:33-35)
        r = 1.0 / UnitSystem.si().unit_of(otype).scale
        return name, func, lo * r, hi * r

    def spec(self, species, units):
        h = abi.HgramSpec()
        h.dim = self.dim
        h.species = species
        for k in range(self.dim):
            h.func[k] = self.funcs[k]
            h.scale[k] = units.unit_of(self.types[k]).scale
        h.weight = WEIGHTS[self.weight]
        h.bin_spec, h.n_bins, h.bin_size = self.bin_spec
        h.height = abi.HEIGHT_DENSITY  # DistributionFunction::load always asks for densities
        if self.filter is None:
            h.filter_func, h.filter_min, h.filter_max = -1, -math.inf, math.inf
        else:
            h.filter_func, h.filter_min, h.filter_max = self.filter[1], self.filter[2], self.filter[3]
        return h

    def suffix(self):
        """output/mod.rs:268-318."""
        s = "_" + "-".join(self.names)
        if self.weight not in ("weight", "auto"):
            s += "_%s-weight" % self.weight
        if self.bin_spec[0] == abi.BINS_LOG:
            s += "_log"
        if self.filter is not None:
            s += "_%s-cut" % self.filter[0]
        return s

    def histogram(self, engine, particles, species, units):
        """(Histogram, or None for an empty set)."""
        info, counts = engine.histogram(particles, self.spec(species, units))
        if counts is None:
            return None
        unit_names = [units.unit_of(t).name for t in self.types]
        return Histogram(info, counts, self.names, unit_names)

    def write(self, engine, particles, species, units, prefix, file_format="plain_text"):
        """Writes prefix + suffix + ".dat" (or ".fits"); returns the file name,
        or None for an empty set."""
        h = self.histogram(engine, particles, species, units)
        if h is None:
            return None
        if file_format == "fits":
            return h.write_fits(prefix + self.suffix())
        return h.write_plain_text(prefix + self.suffix())


VERSION = "0.1.0"


def rust_exp_upper(x, width=20):
    """Rust's `{:>20.9E}`."""
    return rust_exp(x).replace("e", "E").rjust(width)


def rust_exp(x, digits=9):
    """Rust's `{:.9e}` (or another precision) for an f64: the digits after
    the point, an exponent with no sign for positive powers and no padding."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    m, e = ("%.*e" % (digits, x)).split("e")
    return "%se%d" % (m, int(e))


class Histogram:
    """A histogram with the reference's metadata (output/hgram.rs:119-133)."""

    def __init__(self, info, counts, names, units):
        self.dim = info["dim"]
        self.bins = info["bins"]
        self.min, self.max, self.bin_size = info["min"], info["max"], info["bin_size"]
        self.total, self.unweighted_total = info["total"], info["unweighted_total"]
        self.counts = counts
        if self.dim == 1:
            self.name = "hgram/density/%s" % names[0]
            self.bunit = "1/%s" % units[0]
        else:
            self.name = "hgram/density/%s_%s" % (names[0], names[1])
            self.bunit = "1/(%s.%s)" % (units[0], units[1])
        self.axis, self.unit = list(names), list(units)

    def write_fits(self, filename):
        """output/hgram.rs:450-528: a primary HDU of 80-character cards
        padded to 2880 bytes, then the heights as big-endian f64, padded to
        a whole block."""
        cards = ["SIMPLE  = %20s / %-47s" % ("T", "file conforms to FITS standard"),
                 "BITPIX  = %20d / %-47s" % (-64, "number of bits per data pixel"),
                 "NAXIS   = %20d / %-47s" % (self.dim, "number of data axes")]
        for n in range(1, self.dim + 1):
            cards.append("NAXIS%-3d= %20d / %-47s" % (n, self.bins[n - 1], "number of pixels along this axis"))
        cards.append("EXTEND  = %20s / %-47s" % ("T", "dataset may contain extensions"))
        for n in range(1, self.dim + 1):
            cards.append("CRPIX%-3d= %s%-50s" % (n, rust_exp_upper(0.5), ""))
            cards.append("CRVAL%-3d= %s%-50s" % (n, rust_exp_upper(self.min[n - 1]), ""))
            cards.append("CDELT%-3d= %s%-50s" % (n, rust_exp_upper(self.bin_size[n - 1]), ""))
            cards.append("CNAME%-3d= '%s'%s" % (n, self.axis[n - 1], " " * (80 - 12 - len(self.axis[n - 1]))))
            cards.append("CUNIT%-3d= '%s'%s" % (n, self.unit[n - 1], " " * (80 - 12 - len(self.unit[n - 1]))))
        cards.append("BUNIT   = '%s'%s" % (self.bunit, " " * (80 - 12 - len(self.bunit))))
        cards.append("TOTAL   = %s%-50s" % (rust_exp_upper(self.total), ""))
        cards.append("UWTOTAL = %s%-50s" % (rust_exp_upper(self.unweighted_total), ""))
        cards.append("OBJECT  = '%s'%s" % (self.name, " " * (80 - 12 - len(self.name))))
        if len(self.counts):
            lo = hi = float(self.counts[0])
            for c in self.counts:  # the reference's scan (else-if: a new minimum is not tested as a maximum)
                c = float(c)
                if c < lo:
                    lo = c
                elif c > hi:
                    hi = c
            cards.append("DATAMIN = %s%-50s" % (rust_exp_upper(lo), ""))
            cards.append("DATAMAX = %s%-50s" % (rust_exp_upper(hi), ""))
        comment = "COMMENT   Generated by ptarmigan-gb300 v%s" % VERSION
        cards.append(comment.ljust(80))
        cards.append("END".ljust(80))
        header = "".join(cards).encode("ascii")
        if any(len(c) != 80 for c in cards):
            raise ValueError("a FITS card is not 80 characters long")
        header += b" " * ((2880 - len(header) % 2880) % 2880)
        data = np.asarray(self.counts, dtype=">f8").tobytes()
        data += b"\0" * ((2880 - len(data) % 2880) % 2880)
        filename = filename + ".fits"
        with open(filename, "wb") as f:
            f.write(header + data)
        return filename

    def write_plain_text(self, filename):
        """output/hgram.rs:530-562."""
        filename = filename + ".dat"
        lines = ["\t".join(self.axis) + "\t" + self.name, "\t".join(self.unit) + "\t" + self.bunit]
        index = [0] * self.dim
        for ct in self.counts:
            for j in range(self.dim - 1):
                if index[j] >= self.bins[j]:
                    index[j] -= self.bins[j]
                    index[j + 1] += 1
            coord = [self.min[j] + (0.5 + index[j]) * self.bin_size[j] for j in range(self.dim)]
            lines.append("".join(rust_exp(c) + "\t" for c in coord) + rust_exp(float(ct)))
            index[0] += 1
        with open(filename, "w") as f:
            f.write("\n".join(lines) + "\n")
        return filename


# output/stats.rs:19-55
_REDUCTIONS = {"total": "total", "fraction": "fraction", "frac": "fraction", "mean": "mean", "variance": "variance",
               "var": "variance", "minimum": "minimum", "min": "minimum", "maximum": "maximum", "max": "maximum",
               "circmean": "circmean", "cmean": "circmean", "circvariance": "circvar", "cvariance": "circvar",
               "circvar": "circvar", "cvar": "circvar", "circstd": "circstd", "cstd": "circstd"}


class SummaryStatistic:
    """A summary statistic such as "mean energy", "fraction energy in (1e-13;
    auto)" or "variance angle_x`weight for energy in (auto; 1e-12)"
    (SummaryStatistic::load, output/stats.rs:85-262), evaluated on the
    device (ptg_particle_sums).  Bounds are numbers or "auto"."""

    def __init__(self, spec):
        err = ValueError("cannot convert %r to a summary statistic" % spec)
        start, end = spec.find("("), spec.rfind(")")
        rng = spec[start:end + 1] if start >= 0 and end >= 0 else None
        words = (spec.replace(rng, "") if rng else spec).split()
        self.filter = None
        if len(words) == 5:
            if words[2] != "for" or words[3] not in FUNCTIONS:
                raise err
            self.filter = (words[3],) + FUNCTIONS[words[3]]
        lo, hi = -math.inf, math.inf
        if len(words) in (3, 5):
            if rng is None or words[-1] != "in":
                raise err
            parts = ["".join(p.split()) for p in rng[1:-1].split(";")]
            if len(parts) != 2:
                raise err

            def num(t, auto):
                if t == "auto":
                    return auto
                try:
                    return float(t)
                except ValueError:
                    raise err
            lo, hi = num(parts[0], -math.inf), num(parts[1], math.inf)
        if len(words) not in (2, 3, 5) or words[0] not in _REDUCTIONS:
            raise err
        self.op = _REDUCTIONS[words[0]]
        vw = words[1].split("`")
        if len(vw) > 2 or vw[0] not in FUNCTIONS or (len(vw) == 2 and vw[1] not in FUNCTIONS):
            raise err
        self.var_name, self.weight_name = vw[0], (vw[1] if len(vw) == 2 else "unit")
        self.var_func, vtype = FUNCTIONS[self.var_name]
        self.weight_func = FUNCTIONS[self.weight_name][0]
        if self.op in ("circmean", "circvar", "circstd") and vtype != _ANGLE:
            raise err
        unit = UnitSystem.default().unit_of(vtype).name
        if self.op in ("fraction", "circvar"):
            unit = "1"
        elif self.op == "variance":
            unit = "1" if unit == "1" else "(%s)^2" % unit
        self.unit = unit
        if (math.isfinite(lo) or math.isfinite(hi)) and self.filter is None:
            self.filter = (self.var_name, self.var_func, vtype)
        ftype = self.filter[2] if self.filter is not None else vtype
        r = 1.0 / UnitSystem.si().unit_of(ftype).scale  # from_si
        self.min, self.max = lo * r, hi * r
        self.filter_unit = UnitSystem.default().unit_of(self.filter[2]).name if self.filter else None
        self.name, self.value = "", 0.0

    def _spec(self, species, shift=0.0):
        s = abi.StatsSpec()
        s.species, s.var_func, s.weight_func = species, self.var_func, self.weight_func
        s.filter_func = self.filter[1] if self.filter is not None else -1
        s.min, s.max, s.shift = self.min, self.max, shift
        return s

    def evaluate(self, engine, particles, species, name):
        """SummaryStatistic::evaluate (output/stats.rs:412-483)."""
        self.name = name
        a = engine.particle_sums(particles, self._spec(species))
        op = self.op
        if op == "total":
            v = a["subtotal"]
        elif op == "fraction":
            v = a["subtotal"] / a["total"]
        elif op == "mean":
            v = a["subtotal"] / a["count"]
        elif op == "variance":
            # shifted by the mean (the reference shifts by the mean of its
            # first ten particles): the same variance up to rounding
            m = a["subtotal"] / a["count"] if a["count"] else 0.0
            b = engine.particle_sums(particles, self._spec(species, m))
            v = (b["sum_sq_diffs"] - b["sum_diffs"] ** 2 / b["count"]) / b["count"]
        elif op == "minimum":
            v = a["minimum"]
        elif op == "maximum":
            v = a["maximum"]
        else:
            mx, my = a["sum_cos"] / a["count"], a["sum_sin"] / a["count"]
            if op == "circmean":
                v = math.atan2(my, mx)
            elif op == "circvar":
                v = 1.0 - math.hypot(mx, my)
            else:
                v = math.sqrt(-2.0 * math.log(math.hypot(mx, my)))
        self.value = v
        return v

    def __str__(self):
        """impl Display (output/stats.rs:493-516)."""
        bounds = ""
        if self.filter is not None:
            fn, fu = self.filter[0], self.filter_unit
            if math.isfinite(self.min) and math.isinf(self.max):
                bounds = " (%s [%s] > %s)" % (fn, fu, rust_exp(self.min, 6))
            elif math.isinf(self.min) and math.isfinite(self.max):
                bounds = " (%s [%s] < %s)" % (fn, fu, rust_exp(self.max, 6))
            else:
                bounds = " (%s < %s [%s] < %s)" % (rust_exp(self.min, 6), fn, fu, rust_exp(self.max, 6))
        wstr = " (%s-weighted)" % self.weight_name if self.weight_name != "unit" else ""
        return "%s: %s %s%s%s = %s [%s]" % (self.name, self.op, self.var_name, wstr, bounds, rust_exp(self.value, 6),
                                          self.unit)


def write_stats(filename, electron=(), positron=(), photon=()):
    """The stats file of main.rs:1268-1285: electron, then positron, then
    photon statistics, one per line."""
    with open(filename, "w") as f:
        for st in list(electron) + list(positron) + list(photon):
            f.write(str(st) + "\n")
    return filename
