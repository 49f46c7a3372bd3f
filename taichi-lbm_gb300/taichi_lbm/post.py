"""Post-processing (taichi_lbm/PostProcessing.py): normalised field images as
arrays and the legacy ASCII VTK writers.  The reference's interactive
matplotlib plots have no counterpart here (no display on a compute node)."""
import numpy as np


class PostProcessingEngine:
    def __init__(self, num_curves=0):
        self.num_curves = num_curves

    @staticmethod
    def nomalized_field(data):
        """PostProcessing.py:42-46"""
        mn, mx = np.min(data), np.max(data)
        return (data - mn) / (mx - mn)

    def post_pressure(self, lb_field):
        lb_field._sync_fused()
        return self.nomalized_field(lb_field.total_pressure.to_numpy())

    def post_denstiy(self, lb_field):
        lb_field._sync_fused()
        return self.nomalized_field(lb_field.rho.to_numpy()[:, :, 0])

    post_density = post_denstiy

    def post_vel(self, lb_field):
        """PostProcessing.py:64-67"""
        lb_field._sync_fused()
        vel = lb_field.vel.to_numpy()
        return self.nomalized_field((vel[:, :, 0] ** 2.0 + vel[:, :, 1] ** 2.0) ** 0.5)

    def writeVTK(self, fname, lb_field, Tflag=None):
        """ASCII STRUCTURED_GRID with density and velocity (PostProcessing.py:70-120)."""
        lb_field._sync_fused()
        nx, ny = lb_field.NX, lb_field.NY
        rho = lb_field.total_rho.to_numpy().T.flatten()
        vel = lb_field.vel.to_numpy()
        velx, vely = vel[:, :, 0].T.flatten(), vel[:, :, 1].T.flatten()
        xm, ym = np.meshgrid(np.arange(nx), np.arange(ny))
        xf, yf = xm.flatten(), ym.flatten()
        filename = fname + ".vtk"
        with open(filename, "w") as out:
            out.write("# vtk DataFile Version 3.0\nHydrodynamics representation\nASCII\n\n")
            out.write("DATASET STRUCTURED_GRID\n")
            out.write(f"DIMENSIONS {nx} {ny} 1\n")
            out.write(f"POINTS {nx * ny} double\n")
            np.savetxt(out, np.column_stack((xf, yf, np.zeros_like(xf))), fmt="%.0f")
            out.write("\n")
            out.write(f"POINT_DATA {nx * ny}\n")
            out.write("SCALARS density double\nLOOKUP_TABLE density_table\n")
            np.savetxt(out, rho * lb_field.C_rho, fmt="%.8f")
            if Tflag is not None:
                out.write("SCALARS T double\nLOOKUP_TABLE T_table\n")
                np.savetxt(out, lb_field.T.to_numpy().T.flatten(), fmt="%.8f")
            out.write("VECTORS velocity double\n")
            np.savetxt(out, np.column_stack((velx * lb_field.Cu, vely * lb_field.Cu, np.zeros_like(velx))),
                       fmt="%.8f")
        return filename

    def writeVTKpsi(self, fname, lb_field):
        """psi on the haloed grid (PostProcessing.py:123-156)."""
        psi = lb_field.sc_field.psi_field.to_numpy()[:, :, 0].T.flatten()
        nx, ny = lb_field.NX + 2, lb_field.NY + 2
        xm, ym = np.meshgrid(np.arange(nx), np.arange(ny))
        xf, yf = xm.flatten(), ym.flatten()
        filename = fname + ".vtk"
        with open(filename, "w") as out:
            out.write("# vtk DataFile Version 3.0\nHydrodynamics representation\nASCII\n\n")
            out.write("DATASET STRUCTURED_GRID\n")
            out.write(f"DIMENSIONS {nx} {ny} 1\n")
            out.write(f"POINTS {nx * ny} double\n")
            np.savetxt(out, np.column_stack((xf, yf, np.zeros_like(xf))), fmt="%.0f")
            out.write("\n")
            out.write(f"POINT_DATA {nx * ny}\n")
            out.write("SCALARS PSI double\nLOOKUP_TABLE T_table\n")
            np.savetxt(out, psi, fmt="%.8f")
        return filename
