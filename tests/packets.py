"""Test-side SNAP packetiser: builds packet buffers in the reference's format
(MDT_OneStation_client.cu:846-907 reads them) from sample arrays, so that
depacketising must give the arrays back."""
import numpy as np

REF_SNAPS = (10, 10, 10, 8)   # MDT_OneStation_client.h:68
REF_IPS = 38                  # MDT_OneStation_client.h:64


def fmt_dict(sper, bits=32, snaps=REF_SNAPS, ips=REF_IPS, words_header=4):
    per = 8 if bits == 32 else 2
    pb = (4 * words_header + sper * max(snaps) * per + 3) // 4 * 4
    return dict(words_header=words_header, sper_element=sper, inputs_per_station=ips,
                inputs_per_snap=list(snaps), sample_bits=bits, packet_bytes=pb)


def groups(ne, fmt):
    """(station, snap, elem0, nin) of every SNAP whose inputs lie below NE."""
    out = []
    nstation = -(-ne // fmt["inputs_per_station"])
    for st in range(nstation):
        off = st * fmt["inputs_per_station"]
        for k, n in enumerate(fmt["inputs_per_snap"]):
            if off + n <= ne and n > 0:
                out.append((st, k, off, n))
            off += n
    return out


def packetise(words, ne, nch, counters, fmt, grp=None):
    """Packets for `counters` of every group.  words: uint32 [S][NE][Nch][2]
    (32-bit format) or int8 [S][NE][Nch][2] (8-bit), element-samples from 0.
    Returns (uint8 buffer [npkt][packet_bytes], list of (station, snap, counter))."""
    sper = fmt["sper_element"]
    pb = fmt["packet_bytes"]
    hb = 4 * fmt["words_header"]
    flat = words.reshape(-1, ne, nch, 2)
    grp = groups(ne, fmt) if grp is None else grp
    pk = []
    ids = []
    for c in counters:
        idx = c * sper + np.arange(sper)
        spec, chan = idx // nch, idx % nch
        for (st, k, e0, n) in grp:
            buf = np.zeros(pb, np.uint8)
            buf[:12] = np.array([st, k, c], np.uint32).view(np.uint8)
            payload = flat[spec[:, None], e0 + np.arange(n)[None, :], chan[:, None]]  # [sper][n][2]
            raw = np.ascontiguousarray(payload).view(np.uint8).reshape(-1)
            buf[hb:hb + raw.size] = raw
            pk.append(buf)
            ids.append((st, k, c))
    return np.stack(pk) if pk else np.zeros((0, pb), np.uint8), ids


def fixed19(w):
    """The reference's int32 x 2^-19 conversion, vectorised (numpy float64 ->
    float32), including 0x80000000 -> +4096."""
    w = np.asarray(w, np.uint32).astype(np.int64)
    v = np.where(w >= 2 ** 31, w - 2 ** 32, w)
    v = np.where(w == 2 ** 31, 2 ** 31, v)
    return (v.astype(np.float64) * 2.0 ** -19).astype(np.float32)
