"""Reader of the reference call log written by the harness shim (ref_shim.c).

Records: a tag byte, then float64 payload:
  'I' initial FRU set uploaded            (0)
  'V' send_save_state                     (0)
  'R' send_resume_state                   (0)
  'S' distrib_simFRU: st, et, dep0[3], depf[3], Jxfer, Jtr, ICa, Ito2   (12)
  'F' send_calc_fru_flux: dep[3], Jxfer, Jtr, ICa, Ito2                 (7)
  'A' send_calc_fru_avg: state[37], otherstate[12]                      (49)
  'C' fcn with keepc set: time, current[24]                             (25)
  'E' end_mpi                             (0)
"""
import numpy as np

PAYLOAD = {b"I": 0, b"V": 0, b"R": 0, b"E": 0, b"S": 12, b"F": 7, b"A": 49, b"C": 25}


def read_log(path):
    """List of (tag, payload ndarray) in call order."""
    data = open(path, "rb").read()
    out, i = [], 0
    while i < len(data):
        tag = data[i:i + 1]
        n = PAYLOAD[tag]
        i += 1
        out.append((tag.decode(), np.frombuffer(data[i:i + 8 * n], np.float64).copy()))
        i += 8 * n
    return out
