"""The time loop of the reference's model program around the GPU step.

`run` is `ccsm.F90:40-63` with the step replaced by the library: initial mass and
energy, `nsteps` steps of RK4 / RK3_TVD, and at every history time the state handed
to an output callback (the place of `history_write_stat`) and the mass and energy
change ratios (MCR, ECR) printed in the reference's format.  The device keeps the
state between outputs, so the steps between two outputs are one `ccs_step(h, k)`
call (graph replays, no host round trip) instead of the reference's per-step copy.

Time settings follow `parameters_mod.F90`: the namelist group `time_settings`
(:87-92) and its defaults (:118-128), `total_run_time` (:135) and
`nsteps = total_run_time / dt` truncated to an integer (:149).  An output happens
after step `it` when `mod(it*dt, history_interval) == 0` and
`it*dt >= history_interval` (`ccsm.F90:55`), both in double precision as the
reference evaluates them.

The reference computes the energy at an output time from `stat(old)`, the state
before the last step (`ccsm.F90:60`; the mass uses `stat(new)`).  `run` reproduces
that by default; `energy_of_new_state=True` takes the energy of the output state
instead.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable


@dataclass
class TimeSettings:
    """parameters_mod.F90:9-14 with the defaults of :118-128."""
    dt: float = 300.0
    run_days: int = 1
    run_hours: int = 0
    run_minutes: int = 0
    run_seconds: int = 0
    history_interval: int = 360
    integral_scheme: str = "RK4"

    @property
    def total_run_time(self) -> int:
        return self.run_days * 86400 + self.run_hours * 3600 + self.run_minutes * 60 + self.run_seconds

    @property
    def nsteps(self) -> int:
        return int(self.total_run_time / self.dt)

    @property
    def total_output_num(self) -> int:
        return int(self.nsteps * self.dt / self.history_interval)


def _nml_value(tok: str):
    """One namelist value: a quoted string, a logical, an integer or a real (Fortran
    d/D exponents accepted)."""
    t = tok.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1].replace(t[0] * 2, t[0])
    low = t.lower()
    if low in (".true.", ".t.", "t"):
        return True
    if low in (".false.", ".f.", "f"):
        return False
    try:
        return int(t)
    except ValueError:
        return float(low.replace("d", "e"))


def _nml_split(body: str) -> list[str]:
    """The text of one group split at commas and line ends outside quotes, with `!`
    comments removed."""
    out, cur, q = [], [], None
    i = 0
    while i < len(body):
        ch = body[i]
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == "!":
            while i < len(body) and body[i] != "\n":
                i += 1
            continue
        elif ch in ",\n":
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
        i += 1
    out.append("".join(cur))
    return [t for t in (x.strip() for x in out) if t]


def read_namelist(path) -> dict:
    """The groups of a Fortran namelist file (`&group key = value, ... /`) as
    {group: {key: value}}, names lower-cased as Fortran compares them; what
    parameters_mod.F90:readNamelist (:104-113) reads from namelist.input."""
    text = open(path).read()
    groups, i = {}, 0
    while True:
        a = text.find("&", i)
        if a < 0:
            return groups
        e = a + 1
        while e < len(text) and (text[e].isalnum() or text[e] == "_"):
            e += 1
        name = text[a + 1:e].lower()
        # the group ends at the first '/' outside quotes and comments
        j, q, comment = e, None, False
        while j < len(text):
            ch = text[j]
            if comment:
                comment = ch != "\n"
            elif q:
                q = None if ch == q else q
            elif ch in "'\"":
                q = ch
            elif ch == "!":
                comment = True
            elif ch == "/":
                break
            j += 1
        entries, key = {}, None
        for tok in _nml_split(text[e:j]):
            if "=" in tok and not tok.lstrip().startswith(("'", '"')):
                k, v = tok.split("=", 1)
                key = k.strip().lower()
                entries[key] = _nml_value(v) if v.strip() else None
            elif key is not None:  # a continued value list
                prev = entries[key]
                entries[key] = (prev if isinstance(prev, list) else [prev]) + [_nml_value(tok)]
        groups[name] = entries
        i = j + 1


@dataclass
class RunSettings:
    """What the dynamic core's namelist.input selects (parameters_mod.F90:87-100)."""
    time: TimeSettings
    case_num: int = 2
    mesh_file: str = ""
    halo: int = 1            # xhalo (parameters_mod.F90:121; the shipped input sets 4)
    reconstruct_scheme: str = "WENO"


def settings_from_namelist(path) -> RunSettings:
    """RunSettings of a namelist.input, the defaults of parameters_mod.F90:118-128
    for what it leaves out."""
    nml = read_namelist(path)
    ts_g, cs, dom, dyn = (nml.get(g, {}) for g in ("time_settings", "case_select", "domain", "dynamic_opt"))
    ts = TimeSettings(dt=float(ts_g.get("dt", 300.0)), run_days=int(ts_g.get("run_days", 1)),
                      run_hours=int(ts_g.get("run_hours", 0)), run_minutes=int(ts_g.get("run_minutes", 0)),
                      run_seconds=int(ts_g.get("run_seconds", 0)),
                      history_interval=int(ts_g.get("history_interval", 360)),
                      integral_scheme=str(ts_g.get("integral_scheme", "RK4")).strip())
    return RunSettings(ts, int(cs.get("case_num", 2)), str(dom.get("mesh_file", "")).strip(),
                       int(dom.get("xhalo", 1)), str(dyn.get("reconstruct_scheme", "WENO")).strip())


def mesh_resolution_from_namelist(path) -> int:
    """N of the mesh-generation namelist (mesh_generation/src/parameters_mod.f90:40-50):
    dx degrees per cell on a 90-degree panel edge."""
    dom = read_namelist(path).get("domain", {})
    dx = float(dom.get("dx", 1.0))
    n = 90.0 / dx
    if abs(n - round(n)) > 1e-9:
        raise ValueError(f"dx = {dx} degrees does not divide a panel edge")
    return int(round(n))


def output_steps(ts: TimeSettings) -> list[int]:
    """The steps after which ccsm.F90:55 writes output."""
    hi = float(ts.history_interval)
    out = []
    for it in range(1, ts.nsteps + 1):
        t = it * ts.dt
        if math.fmod(t, hi) == 0.0 and t >= hi:
            out.append(it)
    return out


@dataclass
class OutputRecord:
    output_idx: int
    step: int
    mcr: float  # (mass - mass0) / mass0
    ecr: float  # (energy - energy0) / energy0
    courant: float | None = None  # Courant number of the output state (with max_courant)


def run(stepper, ts: TimeSettings, on_output: Callable | None = None, energy_of_new_state: bool = False,
        log: Callable[[str], None] | None = print, check: bool = True,
        max_courant: float | None = None) -> list[OutputRecord]:
    """Advances `stepper` (a model.Stepper whose state is set) through the run of
    `ts`; calls on_output(output_idx, state) at every history time with the state
    as ccs_get_state returns it (sphere winds included); returns the MCR/ECR records.
    With `check`, every output time also runs the health check (ccs_check_state) and
    a state with non-positive depth or non-finite wind stops the run with
    FloatingPointError (the reference has no such check and carries on with NaNs).
    With `max_courant`, every output time also takes the state's Courant number
    (ccs_courant) into its record and stops the run with FloatingPointError above
    that bound (the reference's dt is a namelist constant that nothing checks)."""
    if ts.integral_scheme not in ("RK4", "RK3_TVD"):
        raise ValueError(f"integral_scheme {ts.integral_scheme!r}")
    mass0, energy0 = stepper.diag()
    if on_output is not None:
        on_output(1, stepper.get_state())
    if log:
        log(f" output index/total, MCR, ECR : {0} / {ts.total_output_num}   0.0 0.0")
    records = []
    done = 0
    for k, it in enumerate(output_steps(ts)):
        ahead = it - done
        if energy_of_new_state:
            stepper.step(ahead)
            mass, energy = stepper.diag()
        else:
            if ahead > 1:
                stepper.step(ahead - 1)
            energy = stepper.diag()[1]  # stat(old): the state before step `it`
            stepper.step(1)
            mass = stepper.diag()[0]
        done = it
        idx = k + 2
        if check:
            nbad = stepper.check_state()
            if nbad:
                raise FloatingPointError(f"step {it}: {nbad} cells with non-positive depth or non-finite wind")
        courant = None
        if max_courant is not None:
            courant = stepper.courant()
            if not courant <= max_courant:
                raise FloatingPointError(f"step {it}: Courant number {courant:.4g} above {max_courant}")
        if on_output is not None:
            on_output(idx, stepper.get_state())
        rec = OutputRecord(idx, it, (mass - mass0) / mass0, (energy - energy0) / energy0, courant)
        records.append(rec)
        if log:
            log(f" output index/total, MCR, ECR : {idx - 1} / {ts.total_output_num}   {rec.mcr!r} {rec.ecr!r}")
    if ts.nsteps > done:
        stepper.step(ts.nsteps - done)
    return records


def history_writer(prefix: str, mesh) -> Callable:
    """An on_output callback writing each history state as the checkpoint file
    `prefix_NNNN.ccsstate` (the files `ccsm_gpu --history` writes)."""
    def write(idx, state):
        state.save(f"{prefix}_{idx:04d}.ccsstate", mesh)
    return write


def is_raw_mesh_file(path) -> bool:
    """Whether `path` is a raw-binary mesh file (ccs_mesh_file_info).  The reference's
    own mesh_file is NetCDF (io_mod.F90:37), which cannot be read here: the drivers
    then generate the mesh instead."""
    import ctypes as C

    from . import _lib as L
    fn, fmap = C.c_int(), C.c_int()
    return L.lib().ccs_mesh_file_info(str(path).encode(), C.byref(fn), C.byref(fmap)) == L.CCS_OK


def main(argv=None) -> int:
    """The model program (ccsm.F90) from the reference's namelist files, on the GPU:
    python -m conformal_cubed_sphere_gb300.driver --namelist namelist.input
    [--mesh-namelist FILE | --N N] [--precision fp64|mixed] [--history PREFIX]
    [--max-courant C] [--radius A].  The mesh is generated (conformal cubic map) or
    read from the namelist's mesh_file when that is a raw-binary mesh file."""
    import argparse
    import os

    from . import _lib as L
    from . import model as M

    ap = argparse.ArgumentParser(description="ccsm.F90 time loop on the GPU step")
    ap.add_argument("--namelist", required=True)
    ap.add_argument("--mesh-namelist", default=None)
    ap.add_argument("--N", type=int, default=None)
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--radius", type=float, default=6371229.0)  # constants_mod.F90:9
    ap.add_argument("--history", default=None)
    ap.add_argument("--max-courant", type=float, default=None)
    ap.add_argument("--energy-of-new-state", action="store_true")
    a = ap.parse_args(argv)
    rs = settings_from_namelist(a.namelist)
    if rs.time.integral_scheme not in ("RK4", "RK3_TVD"):
        print(f"unknown integral scheme {rs.time.integral_scheme}")  # parameters_mod.F90:146
        return 2
    raw_mesh = False
    if rs.mesh_file and os.path.exists(rs.mesh_file):
        raw_mesh = is_raw_mesh_file(rs.mesh_file)
        if not raw_mesh:
            print(f" mesh_file {rs.mesh_file} is not a raw-binary mesh file: the mesh is generated")
    if raw_mesh:
        mesh = M.Mesh.from_file(rs.mesh_file, halo=rs.halo, radius=a.radius)
    else:
        N = a.N or (mesh_resolution_from_namelist(a.mesh_namelist) if a.mesh_namelist else None)
        if N is None:
            ap.error("no mesh: give --N or --mesh-namelist (or a raw-binary mesh_file in the namelist)")
        mesh = M.Mesh(N, rs.halo, radius=a.radius)
    kind = {2: L.CCS_IC_CASE2, 5: L.CCS_IC_CASE5, 6: L.CCS_IC_CASE6}.get(rs.case_num)
    if kind is None:
        print(f"unknown case_num {rs.case_num}")
        return 2
    state = M.initial_state(mesh, kind=kind)
    stepper = M.Stepper(mesh, rs.time.dt, precision=a.precision, scheme=rs.time.integral_scheme)
    stepper.set_state(state)
    print(f" Temporal integration scheme is {rs.time.integral_scheme}")
    on_output = history_writer(a.history, mesh) if a.history else None
    try:
        run(stepper, rs.time, on_output=on_output, energy_of_new_state=a.energy_of_new_state,
            max_courant=a.max_courant)
    except FloatingPointError as e:
        print(f"stopped: {e}")
        return 1
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
