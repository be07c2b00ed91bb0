"""Regenerates the golden fixtures in this folder from the Rhyme source tree.

Run once in a container that holds the reference checkout:

    python tests/golden/make_golden.py /path/to/Rhyme

It copies the known-answer DATA the reference's own unit tests read (it
copies no source code):

* p_stars_1000.csv: the first 1000 data rows of
  src/rhyme_riemann_problem/src/rhyme_irs/tests/assets/p_stars.txt, the rows
  rhyme_irs_exec_test.f90:42-57 checks (columns read as left state, right
  state, p*; the file header labels them the other way round, the test reads
  them left first).
* sod_t0.2_analytical.csv: the 500 (x, rho, u, p) rows after the 12-line
  header of src/rhyme_riemann_problem/tests/sod_shock_tube_t_0_2_analytical.txt
  that rhyme_riemann_problem_sampling_test.f90:40-58 compares against.
* toro_star_cases.json: the primitive left/right states and the expected
  star values of Toro's five test problems, parsed from
  src/rhyme_riemann_problem/tests/rhyme_irs_tests_factory.f90:11-184.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def fnum(s):
    return float(s.lower().replace("d", "e"))


def main(root):
    rp = os.path.join(root, "src", "rhyme_riemann_problem")
    # p_stars
    src = os.path.join(rp, "src", "rhyme_irs", "tests", "assets", "p_stars.txt")
    with open(src) as f:
        lines = f.read().splitlines()
    rows = [ln for ln in lines[1:] if ln.strip()][:1000]
    with open(os.path.join(HERE, "p_stars_1000.csv"), "w") as f:
        f.write("# source: rhyme_irs/tests/assets/p_stars.txt rows 1-1000; "
                "columns l_rho,l_v,l_p,r_rho,r_v,r_p,p_star\n")
        f.write("\n".join(rows) + "\n")

    # Sod analytic profile
    src = os.path.join(rp, "tests", "sod_shock_tube_t_0_2_analytical.txt")
    with open(src) as f:
        lines = f.read().splitlines()
    rows = [ln.split() for ln in lines[12:12 + 500]]
    with open(os.path.join(HERE, "sod_t0.2_analytical.csv"), "w") as f:
        f.write("# source: rhyme_riemann_problem/tests/"
                "sod_shock_tube_t_0_2_analytical.txt rows 13-512; "
                "columns x,rho,u,p (gamma=1.4, t=0.2)\n")
        for r in rows:
            f.write(",".join(r[:4]) + "\n")

    # Toro star cases
    src = os.path.join(rp, "tests", "rhyme_irs_tests_factory.f90")
    text = open(src).read()
    cases = []
    for m in re.finditer(r"subroutine (rhyme_riemann_problem_(\w+)_test)\((.*?)end subroutine \1",
                         text, re.S):
        name, body = m.group(2), m.group(3)
        def grab(pat):
            mm = re.search(pat, body)
            return fnum(mm.group(1)) if mm else None
        case = {
            "name": name,
            "left": {"rho": grab(r"l_prim\(cid%rho\) = ([-\d.eEdD+]+)"),
                     "u": grab(r"l_prim\(cid%u\) = ([-\d.eEdD+]+)"),
                     "p": grab(r"l_prim\(cid%p\) = ([-\d.eEdD+]+)")},
            "right": {"rho": grab(r"r_prim\(cid%rho\) = ([-\d.eEdD+]+)"),
                      "u": grab(r"r_prim\(cid%u\) = ([-\d.eEdD+]+)"),
                      "p": grab(r"r_prim\(cid%p\) = ([-\d.eEdD+]+)")},
            "star_p": grab(r"solution%star%p = ([-\d.eEdD+]+)"),
            "star_u": grab(r"solution%star%u = ([-\d.eEdD+]+)"),
            "left_is_shock": ".true." in re.search(r"solution%star%left%is_shock = (\S+)", body).group(1),
            "left_rho": grab(r"solution%star%left%(?:fan|shock)%rho = ([-\d.eEdD+]+)"),
            "right_is_shock": ".true." in re.search(r"solution%star%right%is_shock = (\S+)", body).group(1),
            "right_rho": grab(r"solution%star%right%(?:fan|shock)%rho = ([-\d.eEdD+]+)"),
        }
        cases.append(case)
    sigfig = {"Sod": 6, "123": 4, "left_blast_wave": 6, "right_blast_wave": 6,
              "two_shocks_collision": 3}
    for c in cases:
        c["sig_fig"] = sigfig[c["name"]]
    with open(os.path.join(HERE, "toro_star_cases.json"), "w") as f:
        json.dump({"source": "rhyme_riemann_problem/tests/rhyme_irs_tests_factory.f90:11-184; "
                             "significant figures from rhyme_riemann_problem_star_test.f90:31-35",
                   "gamma": "diatomic (7/5)", "cases": cases}, f, indent=1)
    print("wrote", len(cases), "Toro cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py RHYME_SOURCE_TREE")
    main(sys.argv[1])
