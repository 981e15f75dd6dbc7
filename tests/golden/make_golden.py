"""Regenerates the golden fixtures in tests/golden/ from the reference checkout.

Run where a checkout of the reference is available, giving its root directory:
    python tests/golden/make_golden.py <path to the CaNS checkout>
It copies the reference's own lid-driven-cavity golden v-profile
(tests/lid_driven_cavity/data_ldc_re1000.txt, compared at rtol=1e-7 by the
reference's tests/lid_driven_cavity/test.py:5-8) and records the run
parameters of tests/lid_driven_cavity/input.nml:1-24 that produce it.
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    src = os.path.join(ref, "tests", "lid_driven_cavity", "data_ldc_re1000.txt")
    shutil.copyfile(src, os.path.join(HERE, "ldc_re1000_vprofile.txt"))
    # tests/lid_driven_cavity/input.nml:2-20
    case = dict(ng=[2, 64, 64], l=[0.03125, 1., 1.], gtype=1, gr=0., cfl=0.95, dtmax=1.e5, dt_f=-1.,
                visci=1000., icheck=10, nstep=1500,
                cbcvel="PPDDDD" "PPDDDD" "PPDDDD", cbcpre="PPNNNN",
                bcvel=[0., 0., 0., 0., 0., 0.,
                       0., 0., 0., 0., 0., 1.,
                       0., 0., 0., 0., 0., 0.],
                bcpre=[0.] * 6, bforce=[0.] * 3, is_forced=[0] * 3, velf=[0.] * 3, is_impdiff=0,
                inivel="zer", compare="v(i=1, j=ng2/2+1, k=1..ng3) after nstep steps, rtol 1e-7")
    with open(os.path.join(HERE, "ldc_re1000_case.json"), "w") as f:
        json.dump(case, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the CaNS checkout>")
    main(sys.argv[1])
