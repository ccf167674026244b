"""Text of writer::Atom_writer's output files, restated for the tests.

TEST INFRASTRUCTURE ONLY: used by tests/ to turn the oracle's state into the
files the reference writes, and to compare two such files.  Nothing shipped
imports it.

Formats (the reference streams with std::ostream defaults, i.e. printf "%g" of
precision 6 for doubles):
  xyz          src/writer/atom_writer/dump_xyz_serial.cpp:32-66
               "N\\nAtom\\n", then per atom "type [id] x y z [vx vy vz] [ax ay az]"
  energy etc.  src/writer/atom_writer/dump_energy.cpp: "i t value" per line
  msd          src/writer/atom_writer/dump_msd.cpp:35-101
  schedule     src/writer/atom_writer.cpp:427-466 (output when i % step == 0),
               src/md_simulator.cpp:609-610 (setup writes step 0 at time 0),
               :727-728 (each step writes (current_step, time) before time += dt)
"""
from __future__ import annotations

import numpy as np

KINDS = ("xyz", "energy", "temperature", "pressure", "msd", "volume")


def g6(x):
    """std::ostream << double with default flags (printf %.6g)."""
    return "%.6g" % float(x)


class AtomWriterText:
    """writer::Atom_writer's serial output as strings, fed with host-order state."""

    def __init__(self, cfg, box_size):
        self.cfg = cfg
        self.L = np.asarray(box_size, np.float64)
        self.text = {k: [] for k in KINDS if cfg.get(k, 0) > 0}
        self.msd_initial = None
        self.cross_base = None

    def wants(self, i):
        return any(i % self.cfg[k] == 0 for k in self.text)

    def write(self, i, t, ke, temperature, pressure, pos, vel, acc, typ, cross):
        c = self.cfg
        if "xyz" in self.text and i % c["xyz"] == 0:
            rows = [f"{len(pos)}\nAtom\n"]
            for a in range(len(pos)):
                f = [str(int(typ[a]))]
                if c.get("xyz_id"):
                    f.append(str(a))
                f += [g6(v + 0.0) for v in pos[a]]  # position offset {0,0,0}: -0.0 prints as 0
                if c.get("xyz_velocity"):
                    f += [g6(v) for v in vel[a]]
                if c.get("xyz_acceleration"):
                    f += [g6(v) for v in acc[a]]
                rows.append(" ".join(f) + "\n")
            self.text["xyz"].append("".join(rows))
        for kind, val in (("energy", ke), ("temperature", temperature), ("pressure", pressure),
                          ("volume", float(self.L[0] * self.L[1] * self.L[2]))):
            if kind in self.text and i % c[kind] == 0:
                self.text[kind].append(f"{i} {g6(t)} {g6(val)}\n")
        if "msd" in self.text and i % c["msd"] == 0:
            self._msd(i, t, pos, typ, cross)

    def _msd(self, i, t, pos, typ, cross):
        init = int(self.cfg.get("msd_initial_step", 0))
        if i < init:
            return
        if i == init:  # origin: positions kept, crossing counts zeroed
            self.msd_initial = pos.copy()
            self.cross_base = cross.copy()
            self.text["msd"].append(f"{i} {g6(t)} 0.0\n")
            return
        cr = cross - self.cross_base
        mt = int(self.cfg.get("msd_type", -1))
        s, n, tot = 0.0, 0, [0, 0, 0]
        for j in range(len(pos)):
            if mt > -1 and int(typ[j]) != mt:
                continue
            # the reference's conventions: initial - current + crossings * L, and the
            # y and z totals accumulate the x counts
            dx = self.msd_initial[j, 0] - pos[j, 0]
            dy = self.msd_initial[j, 1] - pos[j, 1]
            dz = self.msd_initial[j, 2] - pos[j, 2]
            dx += cr[j, 0] * self.L[0]
            dy += cr[j, 1] * self.L[1]
            dz += cr[j, 2] * self.L[2]
            tot[0] += int(cr[j, 0])
            tot[1] += int(cr[j, 0])
            tot[2] += int(cr[j, 0])
            s += dx * dx + dy * dy + dz * dz
            n += 1
        msd = s / n if n > 0 else 0.0
        self.text["msd"].append(f"{i} {g6(t)} {g6(msd)} {tot[0]} {tot[1]} {tot[2]} {sum(tot)}\n")

    def files(self):
        return {k: "".join(v) for k, v in self.text.items()}


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return None


def compare_text(mine, ref, rtol=1.1e-5, atol=0.0, what=""):
    """Line and token structure identical; integer tokens identical; float tokens
    equal as text or, where the six-digit rounding of two close values differs,
    within rtol (one unit in the sixth significant digit is 1e-5 relative).
    Returns the number of tokens that differ as text."""
    a, b = mine.splitlines(), ref.splitlines()
    assert len(a) == len(b), f"{what}: {len(a)} lines vs {len(b)}"
    differ = 0
    for ln, (la, lb) in enumerate(zip(a, b)):
        ta, tb = la.split(), lb.split()
        assert len(ta) == len(tb), f"{what}:{ln + 1}: '{la}' vs '{lb}'"
        for x, y in zip(ta, tb):
            if x == y:
                continue
            differ += 1
            fx, fy = _num(x), _num(y)
            assert fx is not None and fy is not None, f"{what}:{ln + 1}: '{x}' vs '{y}'"
            assert "." in x + y or "e" in x + y, f"{what}:{ln + 1}: integer token '{x}' vs '{y}'"
            assert abs(fx - fy) <= rtol * max(abs(fx), abs(fy)) + atol, f"{what}:{ln + 1}: {x} vs {y}"
    return differ
