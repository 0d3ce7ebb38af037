"""Copies the reference's own golden data for the hot path into tests/golden/.

Run once in a checkout that has the reference project (read-only) available:
    python tests/golden/collect_reference_golden.py <path of the reference checkout>

Files (paths inside the reference project):
  test/data/pumas_radiative_moments.csv
      raw DCS energy moments from the official PUMAS C 1.2.3 library
      (pinned by test/test_material_integrals.jl:7-64)
  docs/revision_evidence/corrected_transport/physics-julia.csv
      the reference's own tabulated properties of the revision physics
  examples/data/revision_physics/pumas-materials/dedx/muon/{standard_rock,water,air}.txt
      the PUMAS dE/dx inputs that physics-julia.csv was built from
  docs/revision_evidence/corrected_transport/full102_comparison.csv
      stochastic backward-MC flux (straggling + scattering, 10^4 histories per
      point) of the reference and of the official PUMAS C library on the flat
      rock column: 17 thicknesses x 6 zenith angles
"""
import os
import shutil
import sys

FILES = {
    "test/data/pumas_radiative_moments.csv": "pumas_radiative_moments.csv",
    "docs/revision_evidence/corrected_transport/physics-julia.csv": "physics-julia.csv",
    "examples/data/revision_physics/pumas-materials/dedx/muon/standard_rock.txt": "dedx_muon/standard_rock.txt",
    "examples/data/revision_physics/pumas-materials/dedx/muon/water.txt": "dedx_muon/water.txt",
    "examples/data/revision_physics/pumas-materials/dedx/muon/air.txt": "dedx_muon/air.txt",
    "docs/revision_evidence/corrected_transport/full102_comparison.csv": "full102_comparison.csv",
}


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    for src, dst in FILES.items():
        d = os.path.join(here, dst)
        os.makedirs(os.path.dirname(d), exist_ok=True)
        shutil.copyfile(os.path.join(ref, src), d)
        print(dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
