"""Writes a small FDFK2D input folder (the reference's file formats, src/Input.f90) for the
input/output tests: 40 x 24 grid at 250 m, two-layer crust/mantle, 8-cell PML, P at 6.672 s/deg."""
import os

import numpy as np

NX, NZ, NPML = 40, 24, 8
H = 250.0


def write_folder(d, outsnap=False, nstep=50, tmax=3.0, tstp=0.03, baz_event=(0.0, 140.0), az_org=90.0,
                 pml_top=False):
    """pml_top: the absorbing layer on top (is_PML_top = .true.: the models have npml more rows above
    row 1, and the FK models start above the grid, as the reference requires)."""
    os.makedirs(d, exist_ok=True)
    w = lambda name, text: open(os.path.join(d, name), "w").write(text)
    w("inpar.dat", "FD_model.dat\nSource.dat\nReceiver.dat\nFK_model_left.dat\nFK_model_right.dat\nvp.su\nvs.su\n")
    w("FD_model.dat", "# FD order\n6\n# x0, xn, z0, zn, dx, dz, dt\n0.0 %.1f 0.0 %.1f %.1f %.1f 0.015d0\n"
                      "# tmax, tstp, npml, is_PML_top\n%.3f %.3f %d %s\n# lat_org, lon_org, az_org\n"
                      "30.0, 100.0, %.1f\n# outsnap, nstep\n%s %d\n"
      % ((NX - 1) * H, (NZ - 1) * H, H, H, tmax, tstp, NPML, ".true." if pml_top else ".false.", az_org,
         ".true." if outsnap else ".false.", nstep))
    w("Source.dat", "# f0, ds, src_type\n2.0 1.0e-3 T\n# rayp (s/deg), evla, evlo\n6.672 %.1f %.1f\n" % baz_event)
    rx = [0.0, 1250.0, 4875.0, 7500.0, 9750.0]
    rz = [0.0, 0.0, 1130.0, 0.0, 500.0]
    w("Receiver.dat", "# nrcv\n%d\n# rx rz\n" % len(rx) + "".join("%.1f %.1f\n" % t for t in zip(rx, rz)))
    ztop = -(NPML + 1) * H if pml_top else 0.0
    fk = "# nlayer\n2\n# vp vs ztop\n6300.0 3600.0 %.1f\n8100.0 4500.0 3000.0\n" % ztop
    w("FK_model_left.dat", fk)
    w("FK_model_right.dat", fk)
    top_rows = NPML if pml_top else 0
    NXT, NZT = NX + 2 * NPML, NZ + NPML + top_rows
    z = (np.arange(NZT) - top_rows) * H
    vp = np.where(z < 3000.0, 6300.0, 8100.0).astype(np.float32)
    vs = np.where(z < 3000.0, 3600.0, 4500.0).astype(np.float32)
    head = np.zeros(120, np.int16)
    for name, v in (("vp.su", vp), ("vs.su", vs)):
        with open(os.path.join(d, name), "wb") as f:
            for _ in range(NXT):
                f.write(head.tobytes())
                f.write(v.tobytes())
    return dict(rx=np.array(rx, np.float32), rz=np.array(rz, np.float32))
