"""Copies the reference's own golden outputs and input into this folder.

The reference ships, for each cargo feature set it tests, the res.data and
stdout of one N = 1e7 run at its `valeurs` input (reference/res.data-features_*
and reference/stdout.log-features_*; its CI compares them with numdiff,
.github/workflows/ci.yml:178-203). Symlinked goldens are resolved. Run from
this folder: python make_goldens.py /path/to/3photons-rust
Also writes valeurs_sqrts1000, the valeurs-format input of the sqrt(s) =
1000 GeV configuration (E_min 5 GeV, |cos| cuts 0.95, alpha = 1/137.036,
M_Z = 91.187, Gamma_Z = 2.490, sin^2 theta_W = 0.2315, beta+- = 1, 1e6 events).
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FEATURES = ["", "standard-random", "multi-threading,faster-threading",
            "standard-random,multi-threading,faster-threading", "faster-evgen",
            "no-photon-sorting", "multi-threading", "standard-random,multi-threading", "f32",
            "standard-random,f32"]

SQRTS1000 = """1000000 \t\t\t'Nombre d''evenements'
1000.e0\t\t'energie dans le centre de masse (GeV)'
0.95e0\t\t\t'coupure sur cosinus(photon,faisceau)'
0.95e0\t\t'coupure sur cosinus(photon,photon)'
5.e0 \t\t'coupure sur l''energie (GeV)'
0.e0\t\t\t'coupure sur sinus(normale,faisceau)'
7.2973525205055605e-3\t'constante de structure fine'
7.8125e-3\t\t'constante de structure fine au pic du Z'
0.38937966e9\t\t'facteur de conversion (GeV-2 --> pb)'
91.187e0\t\t'masse du Z (GeV)'
2.490e0                 'largeur du Z (GeV)'
0.2315e0\t\t'sinus carre theta Weinberg'
0.03367e0\t\t'taux de branchement Z--->e+e-'
1.0e0\t\t\t'Beta +'
1.0e0\t\t\t'Beta -'
200\t\t\t'Nombre de bins'
.false.\t\t\t'Impression des resultats ?'
.false.\t\t\t'HBookage des resultats ?'
"""


def main(ref):
    for f in FEATURES:
        for kind in ("res.data", "stdout.log"):
            src = os.path.join(ref, "reference", "%s-features_%s" % (kind, f))
            dst = os.path.join(HERE, "%s-features_%s" % (kind, f.replace(",", "+") or "default"))
            shutil.copyfile(os.path.realpath(src), dst)
    shutil.copyfile(os.path.join(ref, "valeurs"), os.path.join(HERE, "valeurs"))
    with open(os.path.join(HERE, "valeurs_sqrts1000"), "w") as fh:
        fh.write(SQRTS1000)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_goldens.py <path of the reference checkout>")
    main(sys.argv[1])
