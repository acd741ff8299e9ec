"""The benchmark configurations of this path and their seeded synthetic-input
parameters.

No public dataset is involved: every configuration is synthetic int8 I/Q
from the integer generator (mdt_synth_iq / the oracle's synth_iq), whose
per-element noise sigmas, tone tables and source delays are derived here
from the configuration's seed with numpy's PCG64 in double precision and
then frozen as integers (sigma in 1/256 LSB, tones in Q16 LSB, delays in
samples), so the CPU and GPU generators produce identical samples.

  c1_snap10      NE=10,  Nch=1024, Ntaps=4, Nsp=1000, 1 integration; N(0,16^2)
                 per component + tone at FFT channel 137, amplitude 8,
                 per-element random phase.
  c2_station40   NE=40,  Nch=2048, Ntaps=8, Nsp=4096, 16 integrations streamed
                 with PFB history; sigma U[8,24] per element + 3 tones.
  c3_array256    NE=256, Nch=1024, Ntaps=8, Nsp=8192, 8 integrations; 3 point
                 sources (common complex Gaussian streams with integer
                 geometric delays from element positions in a 100 m disk,
                 250 MS/s) in unit receiver noise at SNR 0.1, scaled to
                 sigma 16 LSB before quantisation.
  c5_gaincal64   NE=64,  Nch=512,  Ntaps=4, Nsp=2048, sky as c3.
  (c4: 24 ragged jobs, see ragged_jobs()).
"""
from dataclasses import dataclass, field

import numpy as np

SAMPLE_RATE = 250e6  # samples per second, for geometric delays
C_LIGHT = 299792458.0


@dataclass
class Config:
    name: str
    nelements: int
    nchannels: int
    ntaps: int
    nspectra: int
    nint: int
    seed: int
    kind: str = "tones"         # "tones" or "sky"
    sigma: tuple = (16.0, 16.0)  # uniform range of per-element noise sigma (LSB)
    tones: list = field(default_factory=list)  # [(channel or None, amplitude)]
    nsrc: int = 0
    snr: float = 0.0

    # ------------------------------------------------------------ derived
    def _rng(self, salt):
        return np.random.default_rng([self.seed, salt])

    def sigma_q8(self):
        lo, hi = self.sigma
        if lo == hi:
            s = np.full(self.nelements, lo)
        else:
            s = self._rng(1).uniform(lo, hi, self.nelements)
        return np.round(s * 256).astype(np.int32)

    def tone_channels(self):
        rng = self._rng(2)
        out = []
        for ch, amp in self.tones:
            if ch is None:
                ch = int(rng.integers(1, self.nchannels))
            out.append((ch, amp))
        return out

    def tone_q16(self):
        """Tone table [NE][Nch][2] in Q16 LSB, or None."""
        if not self.tones:
            return None
        rng = self._rng(3)
        c = np.arange(self.nchannels, dtype=np.float64)
        acc = np.zeros((self.nelements, self.nchannels), np.complex128)
        for ch, amp in self.tone_channels():
            phase = rng.uniform(0, 2 * np.pi, self.nelements)
            acc += amp * np.exp(1j * (2 * np.pi * ch * c[None, :] / self.nchannels +
                                      phase[:, None]))
        t = np.stack([acc.real, acc.imag], axis=-1) * 65536.0
        return np.round(t).astype(np.int32)

    def sources(self):
        """(src_sigma_q8[nsrc], src_delay[nsrc][NE]) or (None, None)."""
        if self.nsrc == 0:
            return None, None
        rng = self._rng(4)
        r = 50.0 * np.sqrt(rng.uniform(0, 1, self.nelements))
        th = rng.uniform(0, 2 * np.pi, self.nelements)
        xy = np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
        # source directions: direction cosines inside the unit disk
        lr = np.sqrt(rng.uniform(0, 0.8, self.nsrc))
        lt = rng.uniform(0, 2 * np.pi, self.nsrc)
        lm = np.stack([lr * np.cos(lt), lr * np.sin(lt)], axis=1)
        tau = xy @ lm.T / C_LIGHT * SAMPLE_RATE  # [NE][nsrc] samples
        d = np.round(tau).astype(np.int64)
        d = d - d.min(axis=0, keepdims=True)
        noise = float(np.mean(self.sigma))
        ssig = noise * np.sqrt(self.snr / self.nsrc)
        return (np.full(self.nsrc, round(ssig * 256), np.int32),
                np.ascontiguousarray(d.T.astype(np.int32)))

    def total_spectra(self):
        return self.nint * self.nspectra + self.ntaps - 1

    def antenna_samples(self):
        return self.nelements * self.nspectra * self.nchannels * self.nint


C1 = Config("c1_snap10", 10, 1024, 4, 1000, 1, seed=101, sigma=(16.0, 16.0),
            tones=[(137, 8.0)])
C2 = Config("c2_station40", 40, 2048, 8, 4096, 16, seed=202, sigma=(8.0, 24.0),
            tones=[(None, 8.0), (None, 8.0), (None, 8.0)])
C3 = Config("c3_array256", 256, 1024, 8, 8192, 8, seed=303, kind="sky", sigma=(16.0, 16.0),
            nsrc=3, snr=0.1)
C5 = Config("c5_gaincal64", 64, 512, 4, 2048, 1, seed=505, kind="sky", sigma=(16.0, 16.0),
            nsrc=3, snr=0.1)
CONFIGS = {c.name: c for c in (C1, C2, C3, C5)}


def ragged_jobs(seed=404, njobs=24):
    """Configuration 4: 24 independent jobs of uneven shape."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        jobs.append(Config("c4_job%02d" % j, int(rng.integers(8, 129)),
                           int(rng.choice([512, 1024, 2048])), int(rng.choice([4, 8])),
                           int(rng.integers(256, 8193)), 1, seed=seed * 100 + j,
                           sigma=(float(rng.uniform(8, 24)),) * 2,
                           tones=[(None, 8.0)]))
    return jobs


def small(cfg, nelements=None, nchannels=None, nspectra=None, nint=None, ntaps=None):
    """A reduced copy of a configuration (same generator, smaller sizes)."""
    import dataclasses
    kw = {}
    for k, v in (("nelements", nelements), ("nchannels", nchannels), ("nspectra", nspectra),
                 ("nint", nint), ("ntaps", ntaps)):
        if v is not None:
            kw[k] = v
    c = dataclasses.replace(cfg, **kw)
    if c.tones:
        c.tones = [(None if ch is None or ch >= c.nchannels else ch, a) for ch, a in c.tones]
    return c
