"""Laser descriptions with the reference's constructors and getters.

Mirrors src/Lasers/Cos4Laser.jl, Cos2Laser.jl, GaussianLaser.jl and
BichromaticLaser.jl: the keyword constructors (wave_len or ang_freq,
cyc_num or duration, the Gaussian's three width forms), their checks and
the scalar getters.  Field evaluation happens on the device; these objects
only carry parameters into the C ABI.  Quantities are plain numbers in the
reference's default units (W/cm^2, nm, a.u., rad).
"""
import math
import warnings

from . import abi

_AU_OMEGA_NM = 45.563352525   # omega [a.u.] * lambda [nm] (Cos4Laser.jl:66-68,81)
_INTENSITY_AU = 3.50944521e16  # W/cm^2 per a.u. of intensity (Cos4Laser.jl:85)


class Laser:
    """Supertype of all lasers (Lasers.jl:15)."""


class MonochromaticLaser(Laser):
    """A laser of one carrier frequency (Lasers.jl:21)."""

    def PeakInt(self):
        return self.peak_int

    def WaveLen(self):
        return self.wave_len

    def Ellipticity(self):
        return self.ellip

    def Azimuth(self):
        return self.azi

    def AngFreq(self):
        return _AU_OMEGA_NM / self.wave_len

    def Period(self):
        return 2 * math.pi / self.AngFreq()

    def CEP(self):
        return self.cep

    def TimeShift(self):
        return self.t_shift

    def LaserF0(self):
        return math.sqrt(self.peak_int / (1.0 + self.ellip ** 2) / _INTENSITY_AU)

    def LaserA0(self):
        return self.LaserF0() / self.AngFreq()

    def KeldyshParameter(self, Ip):
        return self.AngFreq() * math.sqrt(2 * Ip) / self.LaserF0()

    def _mono(self, kind, width):
        m = abi.MonoLaser()
        m.kind = kind
        m.peak_int = self.peak_int
        m.wave_len = self.wave_len
        m.cyc_num = width
        m.ellip = self.ellip
        m.azi = self.azi
        m.cep = self.cep
        m.t_shift = self.t_shift
        return m

    def to_c(self):
        L = abi.Laser()
        L.kind = self._kind
        L.mono[0] = self.to_c_mono()
        return L

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__


def _freq_and_wavelen(name, wave_len, ang_freq):
    assert wave_len > 0 or ang_freq > 0, "[%s] Must specify either `wave_len` or `ang_freq`." % name
    if wave_len > 0 and ang_freq > 0:
        warnings.warn("[%s] Both `wave_len` & `ang_freq` are specified, will use `wave_len`." % name)
    if wave_len == 0:
        wave_len = _AU_OMEGA_NM / ang_freq
    else:
        ang_freq = _AU_OMEGA_NM / wave_len
    return wave_len, ang_freq


class _CosNLaser(MonochromaticLaser):
    _name = ""
    _kind = -1

    def __init__(self, peak_int, wave_len=0, ang_freq=0, cyc_num=0, duration=0, ellip=None,
                 azi=0.0, cep=0.0, t_shift=0.0):
        if ellip is None:
            raise TypeError("[%s] `ellip` is required." % self._name)
        wave_len, ang_freq = _freq_and_wavelen(self._name, wave_len, ang_freq)
        assert cyc_num > 0 or duration > 0, \
            "[%s] Must specify either `cyc_num` or `duration`." % self._name
        if cyc_num > 0 and duration > 0:
            warnings.warn("[%s] Both `cyc_num` & `duration` are specified, will use `cyc_num`." % self._name)
        if cyc_num == 0:
            cyc_num = duration / (2 * math.pi / ang_freq)
        self.peak_int = float(peak_int)
        self.wave_len = float(wave_len)
        self.cyc_num = float(cyc_num)
        self.ellip = float(ellip)
        self.azi = float(azi)
        self.cep = float(cep)
        self.t_shift = float(t_shift)

    def Serialize(self):
        """The laser's parameters in the order of Serialize (Cos4Laser.jl:192-204,
        Cos2Laser.jl:192-204)."""
        return {"type": type(self).__name__, "peak_int": self.peak_int, "wave_len": self.wave_len,
                "cyc_num": self.cyc_num, "ellip": self.ellip, "azi": self.azi, "cep": self.cep,
                "t_shift": self.t_shift}

    def CycNum(self):
        return self.cyc_num

    def to_c_mono(self):
        return self._mono(self._kind, self.cyc_num)

    def __repr__(self):
        return "%s(peak_int=%g, wave_len=%g, cyc_num=%g, ellip=%g, azi=%g, cep=%g, t_shift=%g)" % (
            self._name, self.peak_int, self.wave_len, self.cyc_num, self.ellip, self.azi,
            self.cep, self.t_shift)


class Cos4Laser(_CosNLaser):
    """Cos^4-envelope elliptically polarized laser (Cos4Laser.jl:7-74)."""
    _name = "Cos4Laser"
    _kind = abi.LASER_COS4


class Cos2Laser(_CosNLaser):
    """Cos^2-envelope elliptically polarized laser (Cos2Laser.jl:7-74)."""
    _name = "Cos2Laser"
    _kind = abi.LASER_COS2


class GaussianLaser(MonochromaticLaser):
    """Gaussian-envelope elliptically polarized laser (GaussianLaser.jl:7-80)."""
    _name = "GaussianLaser"
    _kind = abi.LASER_GAUSSIAN

    def __init__(self, peak_int, wave_len=0, ang_freq=0, spread_cyc_num=0, spread_duration=0,
                 FWHM_duration=0, ellip=None, azi=0.0, cep=0.0, t_shift=0.0):
        if ellip is None:
            raise TypeError("[GaussianLaser] `ellip` is required.")
        wave_len, ang_freq = _freq_and_wavelen(self._name, wave_len, ang_freq)
        assert spread_cyc_num > 0 or spread_duration > 0 or FWHM_duration > 0, \
            "[GaussianLaser] Must specify one in `spread_cyc_num`, `spread_duration` and `FWHM_duration`."
        if (spread_cyc_num > 0) + (spread_duration > 0) + (FWHM_duration > 0) > 1:
            warnings.warn("[GaussianLaser] More than one in `spread_cyc_num` & `spread_duration` & "
                          "`FWHM_duration` are specified, will use the first positive value.")
        if spread_cyc_num == 0:
            if spread_duration == 0:
                spread_cyc_num = FWHM_duration / (2 * math.sqrt(math.log(2))) / (2 * math.pi / ang_freq)
            else:
                spread_cyc_num = spread_duration / (2 * math.pi / ang_freq)
        self.peak_int = float(peak_int)
        self.wave_len = float(wave_len)
        self.spread_cyc_num = float(spread_cyc_num)
        self.ellip = float(ellip)
        self.azi = float(azi)
        self.cep = float(cep)
        self.t_shift = float(t_shift)

    def Serialize(self):
        """The laser's parameters in the order of Serialize (GaussianLaser.jl:200-212)."""
        return {"type": "GaussianLaser", "peak_int": self.peak_int, "wave_len": self.wave_len,
                "spread_cyc_num": self.spread_cyc_num, "ellip": self.ellip, "azi": self.azi, "cep": self.cep,
                "t_shift": self.t_shift}

    def SpreadCycNum(self):
        return self.spread_cyc_num

    def SpreadDuration(self):
        return self.spread_cyc_num * self.Period()

    def FWHM_Duration(self):
        return self.spread_cyc_num * self.Period() * (2 * math.sqrt(math.log(2)))

    def to_c_mono(self):
        return self._mono(abi.LASER_GAUSSIAN, self.spread_cyc_num)


class BichromaticLaser(Laser):
    """Sum of two monochromatic lasers, the second delayed (BichromaticLaser.jl:7-85)."""

    def __init__(self, l1, l2, delay=0.0):
        if not isinstance(l1, MonochromaticLaser) or not isinstance(l2, MonochromaticLaser):
            raise TypeError("[BichromaticLaser] `l1` and `l2` must be MonochromaticLasers.")
        self.laser1 = l1
        self.laser2 = l2
        self.delay = float(delay)

    def __getitem__(self, i):
        if i == 1:
            return self.laser1
        if i == 2:
            return self.laser2
        raise IndexError("Index of the laser should be either 1 or 2.")

    def Serialize(self):
        """Serialize (BichromaticLaser.jl:101-109): the two lasers' and the delay."""
        return {"type": "BichromaticLaser", "laser1": self.laser1.Serialize(), "laser2": self.laser2.Serialize(),
                "delay21": self.delay}

    def Laser1(self):
        return self.laser1

    def Laser2(self):
        return self.laser2

    def Delay21(self):
        return self.delay

    def to_c(self):
        L = abi.Laser()
        L.kind = abi.LASER_BICHROMATIC
        L.mono[0] = self.laser1.to_c_mono()
        L.mono[1] = self.laser2.to_c_mono()
        L.delay = self.delay
        return L

    def __eq__(self, other):
        return isinstance(other, BichromaticLaser) and self.__dict__ == other.__dict__
