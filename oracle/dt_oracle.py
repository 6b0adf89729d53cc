"""CPU oracle of the reference's dt schedule (test infrastructure only).

DtFrame::Load, radix/SPVSOLVER/MultiGPUSolver/DtFrame.cpp:11-35, restated for files of
whitespace-separated tokens: rows of "Step Dt CourantNumber InflowStep OutputStep" are
read with >> (an int, then four floats) while the stream is good; a row is kept only
if the stream is still good after its fifth field, so reading stops at the first token
that does not parse, at a short last row, and a complete last row not followed by
whitespace is dropped (its last extraction reaches the end of the file).
CMultiGPUHandler::CheckAndUpdateDt, MultiGPUHandler.cpp:1256-1275: one due row per call.
"""
import re

import numpy as np

_INT = re.compile(r"[+-]?\d+$")
_FLT = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def read_dt(text: str):
    toks = text.split()
    trailing_ws = bool(text) and text[-1].isspace()
    rows, i = [], 0
    while i + 5 <= len(toks):
        t = toks[i:i + 5]
        if not _INT.match(t[0]) or not all(_FLT.match(x) for x in t[1:]):
            break
        if i + 5 == len(toks) and not trailing_ws:
            break
        rows.append((int(t[0]), *(float(np.float32(float(x))) for x in t[1:])))
        i += 5
    return rows


def schedule_next(rows, nxt, current_step, param: dict):
    """Returns (next, applied); param holds Dt, CourantNumber, ParticleGenerationStep,
    OutputStep."""
    if 0 <= nxt < len(rows) and current_step >= rows[nxt][0]:
        _, dt, cr, inflow, out = rows[nxt]
        param.update(Dt=dt, CourantNumber=cr, ParticleGenerationStep=int(inflow), OutputStep=int(out))
        return nxt + 1, True
    return nxt, False
