"""Writer of the reference's particle visualisation output (PartVisuFor<RunName>).

Layout, as PIO_Init_visu / PIO_Dump_visu / PIO_Write_XDMF / PIO_Final_visu
write it (src/DEM/Prtcl_IOAndVisu.f90:63-131, 1048-1161, 1166-1263) for one
rank:

- PartVisuFor<RunName><itime I10.10>: binary, native endian, one block per
  field over the particles in their storage order: positions (x, y, z
  float64), then, each when its save_* option is on, id (int32), diameter
  (float64), type (int32), usrMark (int32), linVel(1), linAcc(1), theta,
  rotVel(1), rotAcc(1), contact force, torque (x, y, z float64 each);
- PartVisuFor<RunName>.xmf: an XDMF 2 time series whose grids point into
  those files by byte offset (Seek), written as the reference formats it.

The state comes from sdem_download_particles / a snapshot, the contact force
and torque from sdem_download_forces (or the snapshot's F and T).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from .beds import Particles

RK, IK = 8, 4   # bytes of the reference's real and integer kinds


@dataclass
class VisuOptions:
    """&PrtclVisuOption of the reference's .prm file."""
    saveXDMFOnce: bool = False
    save_ID: bool = True
    save_Diameter: bool = True
    save_Type: bool = True
    save_UsrMark: bool = False
    save_LinVel: bool = True
    save_LinAcc: bool = False
    save_Theta: bool = False
    save_RotVel: bool = True
    save_RotAcc: bool = False
    save_CntctForce: bool = False
    save_Torque: bool = False

    def fields(self):
        """(name, attribute kind, data type, components, bytes per component) of the
        optional blocks in file order."""
        table = [("save_ID", "ID", "Scalar", "Int", 1, IK), ("save_Diameter", "Diameter", "Scalar", "Float", 1, RK),
                 ("save_Type", "Type", "Scalar", "Int", 1, IK), ("save_UsrMark", "UsrMark", "Scalar", "Int", 1, IK),
                 ("save_LinVel", "LinVel", "Vector", "Float", 3, RK),
                 ("save_LinAcc", "LinAcc", "Vector", "Float", 3, RK),
                 ("save_Theta", "Theta", "Vector", "Float", 3, RK),
                 ("save_RotVel", "RotVel", "Vector", "Float", 3, RK),
                 ("save_RotAcc", "RotAcc", "Vector", "Float", 3, RK),
                 ("save_CntctForce", "CntctForce", "Vector", "Float", 3, RK),
                 ("save_Torque", "Torque", "Vector", "Float", 3, RK)]
        return [row[1:] for row in table if getattr(self, row[0])]


class VisuWriter:
    """PIO_Init_visu at construction, PIO_Dump_visu per output step,
    PIO_Final_visu at close().  Output steps are ifirst - 1 + k * save_visu,
    k = 0 .. (ilast - ifirst + 1) // save_visu, as the reference lists them."""

    def __init__(self, res_dir: str, run_name: str, ifirst: int, ilast: int, save_visu: int,
                 options: Optional[VisuOptions] = None, np_in_domain: Optional[int] = None):
        self.dir, self.run, self.opt = res_dir, run_name, options or VisuOptions()
        self.np = np_in_domain
        nflds = (ilast - ifirst + 1) // save_visu + 1
        self.times = [(k - 1) * save_visu + ifirst - 1 for k in range(1, nflds + 1)]
        self.xmf = os.path.join(res_dir, f"PartVisuFor{run_name}.xmf")
        with open(self.xmf, "w") as f:
            f.write('<?xml version="1.0" ?>\n')
            f.write('<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>\n')
            f.write('<Xdmf xmlns:xi="http://www.w3.org/2001/XInclude" Version="2.0">\n')
            f.write('<Domain>\n')
            f.write(' ' * 4 + '<Grid Name="TimeSeries" GridType="Collection" CollectionType="Temporal">\n')
            f.write(' ' * 8 + '<Time TimeType="List">\n')
            f.write(' ' * 12 + f'<DataItem Format="XML" NumberType="Int" Dimensions="{nflds:6d}">\n')
            f.write(' ' * 12 + "".join(f"{t:9d}" for t in self.times))
            f.write(' ' * 12 + '</DataItem>\n')
            f.write(' ' * 8 + '</Time>\n')
        if self.opt.saveXDMFOnce:
            if np_in_domain is None:
                raise ValueError("saveXDMFOnce needs np_in_domain")
            for t in self.times:
                self._grid(t, np_in_domain)
            self._tail()

    def _grid(self, itime: int, n: int) -> None:
        """PIO_Write_XDMF: one grid of the time series."""
        name = f"PartVisuFor{self.run}"
        lines = [' ' * 8 + f'<Grid Name="T{itime:010d}" GridType="Uniform">',
                 ' ' * 12 + f'<Topology TopologyType="Polyvertex" NodesPerElement="{n:9d}"/>',
                 ' ' * 12 + '<Geometry GeometryType="XYZ">',
                 ' ' * 16 + f'<DataItem Format="Binary" DataType="Float" Precision="{RK:1d}" Endian="Native"'
                 f' Dimensions="{3:2d}{n:9d}" Seek="{0:15d}">',
                 ' ' * 20 + f'{name}{itime:010d}',
                 ' ' * 16 + '</DataItem>',
                 ' ' * 12 + '</Geometry>']
        disp = n * 3 * RK
        for fname, kind, dtype, dims, prec in self.opt.fields():
            lines += [' ' * 12 + f'<Attribute Type="{kind}" Center="Node" Name="{fname}">',
                      ' ' * 16 + f'<DataItem Format="Binary" DataType="{dtype}" Precision="{prec:1d}"'
                      f' Endian="Native" Dimensions="{dims:2d}{n:9d}" Seek="{disp:15d}">',
                      ' ' * 20 + f'{name}{itime:010d}',
                      ' ' * 16 + '</DataItem>',
                      ' ' * 12 + '</Attribute>']
            disp += n * dims * prec
        lines.append('        </Grid>')
        with open(self.xmf, "a") as f:
            f.write("\n".join(lines) + "\n")

    def _tail(self) -> None:
        with open(self.xmf, "a") as f:
            f.write('    </Grid>\n</Domain>\n</Xdmf>\n')

    def dump(self, itime: int, p: Particles, F: Optional[np.ndarray] = None, T: Optional[np.ndarray] = None) -> str:
        """PIO_Dump_visu: the binary file of output step itime (and its XDMF
        grid unless saveXDMFOnce); returns the file's path."""
        n = p.n
        if not self.opt.saveXDMFOnce:
            self._grid(itime, n)
        blocks = [np.ascontiguousarray(p.posR[:, :3], np.float64)]
        o = self.opt
        if o.save_ID:
            blocks.append(np.ascontiguousarray(p.id, np.int32))
        if o.save_Diameter:
            blocks.append(2.0 * np.asarray(p.posR[:, 3], np.float64))
        if o.save_Type:
            blocks.append(np.ascontiguousarray(p.ptype, np.int32))
        if o.save_UsrMark:
            blocks.append(np.ascontiguousarray(p.usrmark, np.int32))
        for flag, arr in (("save_LinVel", p.linVel.reshape(n, -1, 3)[:, 0]),
                          ("save_LinAcc", p.linAcc.reshape(n, -1, 3)[:, 0]),
                          ("save_Theta", p.theta), ("save_RotVel", p.rotVel.reshape(n, -1, 3)[:, 0]),
                          ("save_RotAcc", p.rotAcc.reshape(n, -1, 3)[:, 0])):
            if getattr(o, flag):
                blocks.append(np.ascontiguousarray(arr, np.float64))
        for flag, arr in (("save_CntctForce", F), ("save_Torque", T)):
            if getattr(o, flag):
                if arr is None:
                    raise ValueError(f"{flag} needs the forces of the step (sdem_download_forces)")
                blocks.append(np.ascontiguousarray(arr, np.float64).reshape(n, 3))
        path = os.path.join(self.dir, f"PartVisuFor{self.run}{itime:010d}")
        with open(path, "wb") as f:
            for b in blocks:
                b.tofile(f)
        return path

    def close(self) -> None:
        """PIO_Final_visu: the XDMF tail (already written with saveXDMFOnce)."""
        if not self.opt.saveXDMFOnce:
            self._tail()
