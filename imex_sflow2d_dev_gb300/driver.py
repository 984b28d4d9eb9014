"""A run of an IMEX_SfloW2D input file on the GPU: the reference main
program (src/IMEX_SfloW2D.f90) with its time loop on the device.

    python -m imex_sflow2d_dev_gb300.driver [IMEX_SfloW2D.inp] [--fp32]

Sequence (IMEX_SfloW2D.f90 line numbers):
  read_param                         sflow_read_input          (:186-190)
  DEM -> B_cent, B_nodata            sflow_read_dem            (init_grid)
  read_solution (.q_2d restart) or   sflow_read_q2d / sflow_read_restart
    read_restart_file (restart.bin)
  initial output_solution(t)         .q_2d / .p_2d of the start state (:370-371)
  DO WHILE t < t_end:                sflow_advance to the next output time
    ... output_solution(t)           at t >= t_output or t >= t_end (:570-587)
    write_restart_file('restart.bin')
Output names are RUN_NAME_dddd.q_2d / .p_2d with the reference's index
(the restart file's index + 1 for the first output).  Only the outputs the
GPU path supports are written (.q_2d, .p_2d, restart.bin; ESRI, NetCDF,
runout and probe outputs are not), and the output index, t_output and the
dt clamps follow the reference.  Like output_solution, writing the .q_2d
sets |q| < 1e-20 to zero in the state that continues.
"""
import argparse
import os
import sys
import time

import numpy as np

from . import lib as L
from .params import PREC_FP32, PREC_FP64


class Run:
    def __init__(self, input_file, precision=PREC_FP64, workdir=None, verbose=False):
        self.workdir = os.path.abspath(workdir or os.path.dirname(os.path.abspath(input_file)))
        self.verbose = verbose
        p, run = L.read_input(input_file)
        p.precision = precision
        self.p, self.run = p, run
        nx, ny = p.comp_cells_x, p.comp_cells_y
        B, nodata = L.read_dem(self._path(run["topography_file"]), p)
        rf = run["restart_file"]
        self.t = p.t_start
        state = None
        if rf.endswith(".bin"):
            state = L.read_restart(self._path(rf), p)
            q = state["q"]
            B = state["B_cent"]
            self.t = state["t"]
            self.output_idx = 0
        elif rf.split(".")[-1][:3] == "q_2":
            q, self.output_idx = L.read_q2d(self._path(rf), p)
        else:
            raise L.SflowError(-1, f"restart file {rf}: only .q_2d and restart.bin are supported")
        self.B = np.ascontiguousarray(B, dtype=np.float64)
        self.solver = L.Solver(p, self.B)
        if nodata.any():
            self.solver.set_nodata(nodata)   # emptied by every assembly (solver_2d.f90:1626)
        self.solver.upload_q(q)
        if state is not None:
            if p.settling_flag or p.entrainment_flag or p.erosion_coeff != 0.0:
                self.solver.upload_deposit(state["deposit"])
            self.solver.upload_maps(state["hmax"], state["pdynmax"], state["mod_vel_max"])
            self.solver.set_clock(state["t"], state["dt"], state["dt"])
        self.t_output = self.t + p.dt_output
        self.solver.set_output_time(self.t_output)
        self.written = []

    def _path(self, name):
        return name if os.path.isabs(name) else os.path.join(self.workdir, name)

    def output_solution(self, t):
        """output_solution (inpout_2d.f90:5934-6436) for the supported
        outputs, then t_output = t + dt_output."""
        p, run = self.p, self.run
        self.output_idx += 1
        idx = self.output_idx - 1
        if run["output_cons_flag"]:
            q = self.solver.download_q()
            name = self._path(L.output_name(run["run_name"], idx, "q_2d"))
            L.write_q2d(name, p, q)
            self.solver.put_q(q)   # the reference zeroes tiny values in its state
            self.written.append(name)
        if p.topo_change_flag:
            self.B = self.solver.download_topography()
        if run["output_phys_flag"]:
            phys = self.solver.download_phys()
            dep = self.solver.download_deposit()
            h, pd, v = self.solver.maps()
            name = self._path(L.output_name(run["run_name"], idx, "p_2d"))
            L.write_p2d(name, p, phys, self.B, dep, h, pd, v)
            self.written.append(name)
        self.t_output = t + p.dt_output
        self.solver.set_output_time(self.t_output)

    def write_restart(self):
        st = self.solver.stats()
        if self.p.topo_change_flag:
            self.B = self.solver.download_topography()
        h, pd, v = self.solver.maps()
        name = self._path("restart.bin")
        L.write_restart(name, self.p, st.t, st.dt, self.solver.download_q(), self.B,
                        self.solver.download_deposit(), h, pd, v)
        self.written.append(name)

    def log(self, st):
        if self.verbose:
            print(f"t = {st.t:11.4f} dt = {st.dt:9.5f} mass = {st.mass:11.3E} volume = {st.volume:11.3E} "
                  f"area = {st.area:11.3E} solid mass = {st.solid_mass:11.3E}", flush=True)

    def execute(self):
        p, run = self.p, self.run
        any_out = run["output_cons_flag"] or run["output_phys_flag"]
        if any_out:
            self.output_solution(self.t)
        t_wall = time.perf_counter()
        st = self.solver.stats()
        while st.t < p.t_end:
            st = self.solver.advance(t_stop=self.t_output)
            if st.status:
                raise L.SflowError(st.status, f"solver status {st.status:#x} at t = {st.t}")
            self.log(st)
            if st.t >= self.t_output or st.t >= p.t_end:
                if any_out:
                    self.output_solution(st.t)
                    self.write_restart()
                else:
                    self.t_output = st.t + p.dt_output
                    self.solver.set_output_time(self.t_output)
        self.elapsed = time.perf_counter() - t_wall
        return st


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("input", nargs="?", default="IMEX_SfloW2D.inp")
    ap.add_argument("--fp32", action="store_true", help="FP32 bulk form (FP64 Newton)")
    ap.add_argument("--quiet", action="store_true")
    a = ap.parse_args(argv)
    r = Run(a.input, PREC_FP32 if a.fp32 else PREC_FP64, verbose=not a.quiet)
    st = r.execute()
    if not a.quiet:
        print(f"Elapsed real time = {r.elapsed:.3f} seconds, {st.steps} steps; wrote {len(r.written)} files")
    return 0


if __name__ == "__main__":
    sys.exit(main())
