"""Focal-law (``.law``) files: per-shot per-element delays and amplitudes.

Mirrors sim_support/emission_law.py of the reference (``write_law`` :24-67,
``read_law`` :69-113).  The tab-separated format and its nine columns are an
interchange format, so they are reproduced as is::

    # LOIS DE RETARD
    Version 1.0
    numR numS numT numL numV retE ampE retR ampR

``numT`` is the shot, ``numV`` the 1-based element, ``retE``/``ampE`` the
emission delay and gain.  A non-zero ``numS`` marks a full-matrix-capture
file, whose shot count is ``max(numS) + 1``.
"""
import numpy as np

_COLUMNS = ("numR", "numS", "numT", "numL", "numV", "retE", "ampE", "retR", "ampR")


class EmissionLaw:
    def __init__(self):
        for i, name in enumerate(_COLUMNS):
            setattr(self, "_idx_" + name, i)

    @staticmethod
    def _fields(line):
        return line[:-1].split('\t')

    def write_law(self, root, emitter_law, receiver_law=None, emitter_amp=None, reciever_amp=None,
                  elem_range=None):
        """Write ``root + '.law'``; one line per (shot, element)."""
        if elem_range is None:
            elem_range = [0, emitter_law.shape[1] - 1]
        if receiver_law is None:
            receiver_law = emitter_law
        with open(root + ".law", "w") as f:
            f.writelines(["# LOIS DE RETARD \n", "Version 1.0 \n", "\t".join(_COLUMNS) + "\n"])
            for shot in range(emitter_law.shape[0]):
                for e in range(elem_range[0], elem_range[-1] + 1):
                    amp_e = emitter_amp[shot, e] if emitter_amp is not None else 1
                    amp_r = reciever_amp[shot, e] if reciever_amp is not None else 1
                    row = [0, 0, shot, 0, e + 1, emitter_law[shot, e], amp_e, receiver_law[shot, e], amp_r]
                    f.write("\t".join(f"{v}" for v in row) + "\n")

    def read_law(self, file_root):
        """``(delays, amplitudes)``, each ``(n_shots, n_elements)`` float64."""
        with open(file_root) as f:
            lines = f.readlines()
        data = np.array([self._fields(l) for l in lines[3:]], dtype=np.float32)
        n_elem = int(np.max(data[:, self._idx_numV]))
        max_s = int(np.max(data[:, self._idx_numS]))
        n_shots = (max_s if max_s != 0 else int(np.max(data[:, self._idx_numT]))) + 1
        delays = np.zeros((n_shots, n_elem), dtype='float')
        amps = np.zeros((n_shots, n_elem), dtype='float')
        for s in range(n_shots):
            rows = data[s * n_elem:(s + 1) * n_elem]
            delays[s, :] = rows[:, self._idx_retE]
            amps[s, :] = rows[:, self._idx_ampE]
        return delays, amps
