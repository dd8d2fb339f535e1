"""Synthetic radiosonde archives in the two layouts the reference reads (Game/readTable.cpp).

No sounding file ships with the reference, so the tests write their own: seeded ascents
(temperature falling with height, exponential pressure, random humidity and wind) formatted the
way readKNMIFile and readDWDFile parse them. The KNMI layout puts five attributes at token
positions 4..8 of each row line (Pressure, Temperature, Humidity, WindDir, WindSpeed, with the
name lengths the reader skips) and an Altitude attribute elsewhere; the DWD layout is a
';'-separated metadata member listing ascents and a product member holding the rows of many
ascents, in fields 1 (date and hour), 6, 7, 8, 10, 11, 12.

The DWD cases place the target ascent (listed date 161 at 12 UTC) where the reference's
100000-byte stride search behaves differently: in the middle, first in the product member (its
first rows are skipped), last and short (missed), last without a final newline, absent, and with
CRLF line ends.
"""
from __future__ import annotations

import datetime as _dt
import io
import os
import zipfile

import numpy as np

STATION = "04711"
DWD_ARCHIVE = f"synthetic_aero_{STATION}_ascents.zip"
DWD_CASES = ("mid", "first", "tail", "tail_short", "tail_noeol", "missing", "crlf", "coarse")
KNMI_CASES = ("fine", "coarse", "exact", "burst")


def _profile(rng, h0, dz, rows, jitter=True):
    k = np.arange(rows, dtype=np.float64)
    h = h0 + k * dz
    if jitter:
        h = h + rng.uniform(0.0, 0.4 * dz, rows)
        h[0] = h0
    t_k = 291.0 - 0.0065 * (h - h0) + rng.normal(0.0, 0.15, rows)
    p = 1012.7 * np.exp(-(h - h0) / 8150.0)
    rh = np.clip(85.0 - 0.008 * (h - h0) + rng.normal(0.0, 6.0, rows), 3.0, 100.0)
    dd = rng.uniform(0.0, 360.0, rows)
    ff = np.abs(4.0 + 0.004 * (h - h0) + rng.normal(0.0, 1.5, rows))
    return h, t_k, p, rh, dd, ff


def knmi_text(case: str, seed: int) -> str:
    rng = np.random.default_rng(seed)
    h0 = 19.5
    if case == "coarse":
        h, t_k, p, rh, dd, ff = _profile(rng, h0, 157.0, 60)
    elif case == "exact":  # rows every 2 m: levels at multiples of 2 m fall exactly on rows
        h, t_k, p, rh, dd, ff = _profile(rng, h0, 2.0, 2100, jitter=False)
    else:
        h, t_k, p, rh, dd, ff = _profile(rng, h0, 5.0, 1000)
    lines = ['<?xml version="1.0" encoding="utf-8"?><SynchronizedSoundingData>']
    n = h.size
    drop = np.zeros(n, bool)
    if case == "burst":  # the balloon bursts: the last rows come down again
        h = np.concatenate([h, h[-1] - np.arange(1, 8) * 9.0])
        extra = lambda a: np.concatenate([a, a[-7:][::-1]])
        t_k, p, rh, dd, ff = (extra(a) for a in (t_k, p, rh, dd, ff))
        drop = np.concatenate([drop, np.ones(7, bool)])
    for k in range(h.size):
        lines.append(f'<Row Index="{k}" Time="{k * 1.0:.1f}" Flags="0" Pressure="{p[k]:.2f}" '
                     f'Temperature="{t_k[k]:.2f}" Humidity="{rh[k]:.1f}" WindDir="{dd[k]:.1f}" '
                     f'WindSpeed="{ff[k]:.2f}" Altitude="{h[k]:.2f}" Dropping="{int(drop[k])}" />')
    lines.append("</SynchronizedSoundingData>")
    return "\n".join(lines) + "\n"


def knmi_archive(case: str, seed: int) -> bytes:
    """The .mwx archive (a zip) of one KNMI case, in memory."""
    buf = io.BytesIO()
    with zipfile.ZipFile(buf, "w", zipfile.ZIP_DEFLATED) as zf:
        zf.writestr("SynchronizedSoundingData.xml", knmi_text(case, seed))
        zf.writestr("Manifest.xml", "<Manifest />\n")
    return buf.getvalue()


def write_knmi(directory: str, case: str, seed: int) -> str:
    path = os.path.join(directory, f"synthetic_{case}_{seed}.mwx")
    with open(path, "wb") as f:
        f.write(knmi_archive(case, seed))
    return path


def _dates(n=200):
    d0 = _dt.date(2024, 1, 1)
    return [(d0 + _dt.timedelta(days=k)).strftime("%Y%m%d") for k in range(n)]


def dwd_members(case: str, seed: int):
    """(metadata name, metadata text, product name, product text) for one DWD case."""
    rng = np.random.default_rng(seed)
    dates = _dates()
    st = int(STATION)
    meta = ["Stations_ID;Datum;Geogr.Breite;Geogr.Laenge;Stationshoehe;Typ;Sonde;Bodendruck;Bodentemperatur;eor"]
    for d in dates:
        meta.append(f"{st};{d}12;52.10;5.18;{rng.uniform(5, 60):.1f};RS41;X;{rng.uniform(990, 1030):.1f};"
                    f"{rng.uniform(-5, 30):.1f};eor")
    target = dates[161]
    two = ("00", "12")
    before = [(dates[k], 900, two) for k in (157, 158, 159, 160)]
    after = [(dates[k], 900, two) for k in (162, 163, 164)]
    if case == "first":  # the target's 12 UTC rows open the product member
        ascents = [(target, 900, ("12",))] + after
    elif case == "tail":
        ascents = before + [(target, 300, two)]
    elif case == "tail_short":
        ascents = before + [(target, 40, two)]
    elif case == "tail_noeol":
        ascents = before + [(target, 1600, two)]
    elif case == "missing":
        ascents = before + after
    else:
        ascents = before[1:] + [(target, 1400 if case == "coarse" else 900, two)] + after[:2]
    rows = ["Stations_ID;Datum;Sekunde;Geogr.Breite;Geogr.Laenge;Qualitaet;Hoehe;Druck;Temperatur;Feuchte;"
            "Taupunkt;Windgeschwindigkeit;Windrichtung;eor"]
    for d, n, hours in ascents:
        for hh in hours:
            dz = 3.0 if case == "coarse" else 5.0
            h, t_k, p, rh, dd, ff = _profile(rng, float(rng.uniform(40, 90)), dz, n)
            t_c = t_k - 273.15
            td = t_c - (100.0 - rh) / 5.0
            for k in range(n):
                rows.append(f"{st:6d};{d}{hh};{k:5d};52.10;5.18;3;{h[k]:.1f};{p[k]:.2f};{t_c[k]:.1f};{rh[k]:.1f};"
                            f"{td[k]:.1f};{ff[k]:.1f};{dd[k]:.0f};eor")
    eol = "\r\n" if case == "crlf" else "\n"
    meta_text = eol.join(meta) + eol
    prod_text = eol.join(rows) + ("" if case == "tail_noeol" else eol)  # the target ascent ends "tail_noeol"
    meta_name = f"Metadaten_Sekunde_Aero_{STATION}.txt"
    prod_name = f"produkt_sec_aero_{dates[0]}_{dates[-1]}_{STATION}.txt"
    return meta_name, meta_text, prod_name, prod_text


def dwd_archive(case: str, seed: int) -> bytes:
    """The zip archive of one DWD case, in memory (its file name is DWD_ARCHIVE)."""
    meta_name, meta_text, prod_name, prod_text = dwd_members(case, seed)
    buf = io.BytesIO()
    with zipfile.ZipFile(buf, "w", zipfile.ZIP_DEFLATED) as zf:
        zf.writestr(meta_name, meta_text)
        zf.writestr(prod_name, prod_text)
    return buf.getvalue()


def write_dwd(directory: str, case: str, seed: int) -> str:
    """Write the archive into ``directory``; returns its file name (the reader's station field)."""
    with open(os.path.join(directory, DWD_ARCHIVE), "wb") as f:
        f.write(dwd_archive(case, seed))
    return DWD_ARCHIVE
