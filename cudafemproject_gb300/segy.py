"""Receiver traces of a dynamic run -> SEG-Y rev. 1 files.

Writes what the reference's trace converter writes
(FEMproject/segyUtils/src/segyUtils.cpp:11-217, with the segyio2 C library
of FEMproject/thirdparty/segyio2 underneath), byte for byte:

* the receiver text file it reads (VTKfile/src/VTKfile.cpp:72-87 and the
  header lines of femfunc/src/femfunc.cpp:233-238): ``count<TAB>id<TAB>...``,
  then per time sample ``t v1 v2 ...`` in the default C++ stream format
  (``%g``, six significant digits);
* a 3200-byte EBCDIC text header of 40 cards naming the program, the
  receiver quantity ("Displacement Along X" ...), the date, the element /
  node / sample counts and the first / last sample and the interval in ms.
  The reference's first card is 82 characters wide, so the later cards and
  the fields written into them sit 2 characters later and the header is cut
  at 3200 bytes; kept as is, so that files match;
* a 400-byte binary header (big-endian): traces, sample interval in us (in ms
  when it exceeds 32767), samples per trace, format 1 (4-byte IBM float),
  sorting code 4, metres, SEG-Y revision 1, fixed-length traces;
* per trace a 240-byte header (source / group / CDP x = receiver x and the
  source-surface / receiver-group elevations = receiver y, both truncated to
  integers; coordinate units 1; sample count and interval; inline = node id;
  crossline 1; source type = axis + 1) and its samples as big-endian IBM
  floats.

IBM floats are sign | 7-bit base-16 exponent biased by 64 | 24-bit fraction.
The reference converts IEEE floats by shifting the 24-bit significand right
by 0-3 bits to align the exponent to a multiple of four, truncating the bits
shifted out; zeros of either sign become 0 and subnormals are converted as if
normal. ``ibm_from_float`` does the same from that definition.
"""
from __future__ import annotations

import time as _time
from typing import Optional, Sequence

import numpy as np

# ReceiversType (Tools/src/Tools.h:40-49) and its info names (Tools/src/Tools.cpp:35-79)
DISPLACEMENT, VELOCITY, PRINCIPAL_STRESS, PRESSURE, ACCELERATION = 0, 1, 2, 3, 4
_QUANTITY = {DISPLACEMENT: "Displacement", VELOCITY: "Velocity", PRINCIPAL_STRESS: "Principal Stress",
             ACCELERATION: "Acceleration"}

# 1-based byte positions and sizes (SEG-Y rev. 1): binary header fields in the file,
# trace header fields within the 240-byte trace header
BIN_FIELDS = {"traces": (3213, 2), "interval": (3217, 2), "samples": (3221, 2), "format": (3225, 2),
              "sorting": (3229, 2), "measurement": (3255, 2), "revision": (3501, 2), "fixed_length": (3503, 2)}
TRACE_FIELDS = {"recv_group_elev": (41, 4), "source_surf_elev": (45, 4), "source_x": (73, 4), "group_x": (81, 4),
                "coord_units": (89, 2), "sample_count": (115, 2), "sample_inter": (117, 2), "cdp_x": (181, 4),
                "inline": (189, 4), "crossline": (193, 4), "source_type": (217, 2)}

_CARDS = ["C 1 PROGRAM: CudaFEMproject", "C 2 LICENSE:", "C 3 CLIENT:", "C 4 RECORDING PARAMETER:",
          "C 5 FILE FORMAT: SEG-Y Rev.1", "C 6 DATE:", "C 7 NUMBER OF ELEMENTS IN CALCULATED MODEL:",
          "C 8 NUMBER OF NODES IN CALCULATED MODEL:", "C 9 NUMBER OF SAMPLES IN TRACE:", "C10",
          "C11 FIRST SAMPLE:", "C12 LAST SAMPLE:", "C13 SAMPLE INTERVAL:", "C14", "C15 TRACE HEADER POSITION:",
          "C16 OFFSET BYTES 037-041", "C17 INLINE BYTES 189-193", "C18 CROSSLINE BYTES 193-197", "C19",
          "C20 END EBCDIC HEADER"] + [f"C{k}" for k in range(21, 41)]
_FIRST_CARD_WIDTH = 82

_DAYS = ("Mon", "Tue", "Wed", "Thu", "Fri", "Sat", "Sun")
_MONTHS = ("Jan", "Feb", "Mar", "Apr", "May", "Jun", "Jul", "Aug", "Sep", "Oct", "Nov", "Dec")


def quantity_name(quantity: int, dof: int) -> str:
    """ReceiversTypeToInfoName (Tools/src/Tools.cpp:35-79)."""
    if quantity == PRESSURE:
        return "Pressure"
    if quantity in _QUANTITY and 0 <= dof <= 2:
        return f"{_QUANTITY[quantity]} Along {'XYZ'[dof]}"
    return "Undefined"


def ctime_string(t: Optional[float] = None) -> str:
    """The local time as std::ctime prints it, without the newline ("Thu Dec  3 10:04:05 2026")."""
    tm = _time.localtime(t)
    return (f"{_DAYS[tm.tm_wday]} {_MONTHS[tm.tm_mon - 1]} {tm.tm_mday:2d} "
            f"{tm.tm_hour:02d}:{tm.tm_min:02d}:{tm.tm_sec:02d} {tm.tm_year}")


# ----------------------------------------------------------------------------- receiver text files

def write_receiver_text(path: str, node_ids: Sequence[int], times: Sequence[float], traces) -> None:
    """Receiver text file of traces [n_samples][n_traces] (FP32 values, %g)."""
    node_ids = [int(i) for i in node_ids]
    tr = np.asarray(traces, dtype=np.float32).reshape(len(times), len(node_ids))
    t32 = np.asarray(times, dtype=np.float32)
    with open(path, "w") as f:
        f.write(f"{len(node_ids)}\t" + "".join(f"{i}\t" for i in node_ids) + "\n")
        for t, row in zip(t32, tr):
            f.write(f"{float(t):g} " + "".join(f"{float(v):g} " for v in row) + "\n")


def read_receiver_text(path: str):
    """(node_ids, times, traces [n_samples][n_traces]) as float32, read the way
    fill_sgy_with_traces does (segyUtils.cpp:95-123): the first line holds the
    trace count and the node ids, every further line a time and one value per trace."""
    with open(path) as f:
        head = f.readline().split()
        n = int(head[0])
        ids = [int(v) for v in head[1:1 + n]]
        times, rows = [], []
        for line in f:
            tok = line.split()
            if not tok:
                continue
            times.append(float(tok[0]))
            rows.append([float(v) for v in tok[1:1 + n]])
    if any(len(r) != n for r in rows):
        raise ValueError(f"{path}: every sample line needs a time and {n} trace values")
    return ids, np.array(times, dtype=np.float32), np.array(rows, dtype=np.float32).reshape(len(rows), n)


# ----------------------------------------------------------------------------- encoding

def ibm_from_float(values) -> bytes:
    """IEEE float32 values -> big-endian 4-byte IBM floats (truncating, as the reference does)."""
    bits = np.ascontiguousarray(values, dtype=np.float32).reshape(-1).view(np.uint32).astype(np.uint64)
    sign = bits & 0x80000000
    e = (bits >> 23) & 0xFF
    sig = (bits & 0x7FFFFF) | 0x800000                 # value = sig * 2**(e - 150)
    shift = (2 - e) % 4                                # value = (sig >> shift) * 16**(x - 64) * 2**-24
    x = (e + 130 + shift) // 4
    word = sign | (x << 24) | (sig >> shift)
    word = np.where(bits & 0x7FFFFFFF, word, 0)
    return word.astype(">u4").tobytes()


def float_from_ibm(data: bytes) -> np.ndarray:
    """Big-endian IBM floats -> float64 (exact)."""
    w = np.frombuffer(data, dtype=">u4").astype(np.int64)
    frac = (w & 0xFFFFFF).astype(np.float64) * 2.0 ** -24
    val = np.ldexp(frac, 4 * (((w >> 24) & 0x7F) - 64))
    return np.where(w & 0x80000000, -val, val)


def _ebcdic(text: bytes) -> bytes:
    """ASCII -> EBCDIC code page 037 (the header holds letters, digits, space, '.', ':', '-' and NUL)."""
    return text.decode("latin-1").encode("cp037")


def _ceil_scaled(t: float, scale: float) -> int:
    """int(t * scale) plus one when t * scale has a fractional part (segyUtils.cpp:74-80)."""
    v = int(t * scale)
    return v + (1 if t * scale - v > 0 else 0)


def text_header(times, quantity: int, dof: int, n_elems: int, n_nodes: int, date: Optional[str] = None) -> bytes:
    """The 3200-byte text header, EBCDIC (getLineTextHeader, segyUtils.cpp:12-88)."""
    cards = [_CARDS[0].ljust(_FIRST_CARD_WIDTH)] + [c.ljust(80) for c in _CARDS[1:]]
    buf = bytearray("".join(cards).encode("ascii"))
    buf[-1] = 0x80                                     # the last card ends in 0x80 (cut off below)

    def put(card: int, col: int, s: str) -> None:      # NUL-terminated, at card * 80 + col
        b = s.encode("ascii") + b"\0"
        buf[card * 80 + col:card * 80 + col + len(b)] = b

    t32 = [float(np.float32(t)) for t in times]
    put(0, 25, "1.0")
    put(1, 13, "Unprotected")
    put(2, 12, "CudaFEMproject")
    put(3, 25, quantity_name(quantity, dof))
    put(5, 10, ctime_string() if date is None else date)
    put(6, 44, str(int(n_elems)))
    put(7, 41, str(int(n_nodes)))
    put(8, 33, str(len(t32)))
    if t32:
        first = f"{_ceil_scaled(t32[0], 1e3)} MS"
        put(10, 18, first)
        put(11, 17, f"{_ceil_scaled(t32[-1], 1e3)} MS")
        put(12, 21, first)
    return _ebcdic(bytes(buf[:3200]))


def sample_interval(times) -> int:
    """Sample interval of the headers: the first sample time in us, rounded up,
    in ms when above 32767 us (segyUtils.cpp:136-146)."""
    if len(times) == 0:
        return 0
    t0 = float(np.float32(times[0]))
    v = int(t0 * 1e6)
    v += 1 if t0 * 1e6 - float(np.float32(v)) > 0 else 0
    return v // 1000 if v > 32767 else v


def _put(buf: bytearray, pos: int, size: int, value: int) -> None:
    buf[pos - 1:pos - 1 + size] = (int(value) & ((1 << (8 * size)) - 1)).to_bytes(size, "big")


def _coord(v) -> int:
    """static_cast<int> of a single-precision coordinate."""
    return int(np.float32(v))


def write_segy(path: str, node_ids: Sequence[int], times, traces, nodes, dof: int, n_elems: int,
               quantity: int = DISPLACEMENT, date: Optional[str] = None) -> None:
    """SEG-Y file of receiver traces [n_samples][n_traces] recorded at node_ids.

    nodes [n_nodes][dim] gives the receiver coordinates, dof the recorded axis
    (0 x, 1 y, 2 z), quantity the receiver type (DISPLACEMENT, VELOCITY, ...);
    date replaces the current time in the text header."""
    node_ids = [int(i) for i in node_ids]
    nodes = np.asarray(nodes)
    tr = np.asarray(traces, dtype=np.float32).reshape(len(times), len(node_ids))
    ns = len(times)
    interval = sample_interval(times)
    binh = bytearray(400)
    for key, val in (("traces", len(node_ids)), ("interval", interval), ("samples", ns), ("format", 1),
                     ("revision", 1), ("sorting", 4), ("measurement", 1), ("fixed_length", 1)):
        pos, size = BIN_FIELDS[key]
        _put(binh, pos - 3200, size, val)
    out = [text_header(times, quantity, dof, n_elems, len(nodes), date), bytes(binh)]
    for i, nid in enumerate(node_ids):
        if not 0 <= nid < len(nodes):
            raise ValueError(f"receiver node {nid} out of range")
        th = bytearray(240)
        x, y = _coord(nodes[nid][0]), _coord(nodes[nid][1])
        for key, val in (("source_x", x), ("group_x", x), ("cdp_x", x), ("recv_group_elev", y),
                         ("source_surf_elev", y), ("coord_units", 1), ("sample_count", ns),
                         ("sample_inter", interval), ("inline", nid), ("crossline", 1), ("source_type", dof + 1)):
            pos, size = TRACE_FIELDS[key]
            _put(th, pos, size, val)
        out += [bytes(th), ibm_from_float(tr[:, i])]
    with open(path, "wb") as f:
        f.write(b"".join(out))


def convert(out_path: str, txt_path: str, quantity: int, nodes, dof: int, n_elems: int,
            date: Optional[str] = None) -> None:
    """convert() of segyUtils.cpp:197-217: receiver text file -> SEG-Y file."""
    ids, times, traces = read_receiver_text(txt_path)
    write_segy(out_path, ids, times, traces, nodes, dof, n_elems, quantity, date)


def traces_to_segy(path: str, nodes, n_elems: int, receivers: Sequence[int], dt: float, trace, dof: int,
                   quantity: int = DISPLACEMENT, date: Optional[str] = None) -> None:
    """SEG-Y of the traces a dynamic solve recorded ([steps][n_receivers][dim],
    the receiver_trace buffer of cfem_dyn): sample k is time (k + 1) * dt, the
    time of step k + 1 of the reference's loop (femfunc.cpp:245-247)."""
    trace = np.asarray(trace)
    times = (np.arange(1, trace.shape[0] + 1, dtype=np.float32) * np.float32(dt)).astype(np.float32)
    write_segy(path, receivers, times, trace[:, :, dof], nodes, dof, n_elems, quantity, date)


def read_segy(path: str):
    """(text header as ASCII, binary header fields, [(trace header fields, samples float64)])."""
    data = open(path, "rb").read()
    get = lambda b, pos, size: int.from_bytes(b[pos - 1:pos - 1 + size], "big", signed=True)
    text = data[:3200].decode("cp037")
    bh = {k: get(data, p, s) for k, (p, s) in BIN_FIELDS.items()}
    ns = bh["samples"]
    traces = []
    off = 3600
    while off + 240 <= len(data):
        th = data[off:off + 240]
        traces.append(({k: get(th, p, s) for k, (p, s) in TRACE_FIELDS.items()},
                       float_from_ibm(data[off + 240:off + 240 + 4 * ns])))
        off += 240 + 4 * ns
    return text, bh, traces
