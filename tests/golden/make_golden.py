"""Extract the reference's known-answer values into notebook_pins.json.

The reference (heyoka.py) cannot be run here, so its only outputs are the
ones recorded in its documentation notebooks.  This script reads those
notebooks from a heyoka.py source tree and writes the numbers that pin the
batch integrator (step sizes, step counts, min/max step, states, dense and
continuous output) to ``notebook_pins.json`` next to this file.  The tests
read only the JSON.

Usage: python tests/golden/make_golden.py /path/to/heyoka.py
"""

import json
import os
import re
import sys

NUM = r"-?\d+\.\d+(?:e[-+]?\d+)?|-?\d+(?:e[-+]?\d+)?"


def cells(path):
    nb = json.load(open(path))
    out = []
    for c in nb["cells"]:
        txt = ""
        for o in c.get("outputs", []):
            t = o.get("text") or o.get("data", {}).get("text/plain")
            if t:
                txt += "".join(t)
        out.append(("".join(c["source"]), txt))
    return out


def find(cs, needle, exact=False):
    for src, out in cs:
        if (src.strip() == needle) if exact else (needle in src):
            return out
    raise KeyError(needle)


def nums(s):
    return [float(x) for x in re.findall(NUM, s)]


def main(root):
    nbdir = os.path.join(root, "doc", "notebooks")
    pins = {"source": "heyoka.py documentation notebooks (doc/notebooks)"}

    # ---- scalar pendulum, doc/notebooks/The adaptive integrator.ipynb
    cs = cells(os.path.join(nbdir, "The adaptive integrator.ipynb"))
    pins["pendulum"] = p = {"ic": [0.05, 0.025], "order": int(re.search(r"Taylor order\s*:\s*(\d+)", cs[1][1]).group(1))}
    p["first_h"] = float(re.search(r"Timestep: (" + NUM + ")", find(cs, "oc, h = ta.step()\n")).group(1))
    p["back_h"] = float(re.search(r"Timestep: (" + NUM + ")", find(cs, "ta.step_backward()")).group(1))
    out = find(cs, 'print("Current time        : {}".format(ta.time))')
    m = re.search(r"Current time\s*: (" + NUM + r")\nCurrent state vector: \[(.*?)\]", out)
    p["after_clamped_steps"] = {"time": float(m.group(1)), "state_8digits": nums(m.group(2))}
    out = find(cs, "ta.propagate_for(delta_t=5.0)")
    blocks = re.findall(r"Min\. timestep: (" + NUM + r")\nMax\. timestep: (" + NUM + r")\nNum\. of steps: (\d+)", out)
    p["for5"] = {"min_h": float(blocks[0][0]), "max_h": float(blocks[0][1]), "n_steps": int(blocks[0][2])}
    p["until20"] = {"min_h": float(blocks[1][0]), "max_h": float(blocks[1][1]), "n_steps": int(blocks[1][2])}
    out = find(cs, "# Propagate back to t = 0.")
    b = re.findall(r"Min\. timestep: (" + NUM + r")\nMax\. timestep: (" + NUM + r")\nNum\. of steps: (\d+)", out)[0]
    st = re.search(r"State\s*: \[(.*?)\]", out).group(1)
    p["until0"] = {"min_h": float(b[0]), "max_h": float(b[1]), "n_steps": int(b[2]), "state": nums(st)}
    out = find(cs, "out = ta.propagate_grid(grid=[0.0, 0.1")
    m = re.search(r"-4294967299>,\s*(" + NUM + r"),\s*(" + NUM + r"),\s*(\d+),", out)
    rows = re.findall(r"\[\s*(" + NUM + r")\s*,\s*(" + NUM + r")\s*\]", out)
    p["grid"] = {
        "grid": [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0],
        "min_h": float(m.group(1)),
        "max_h": float(m.group(2)),
        "n_steps": int(m.group(3)),
        "out_8digits": [[float(a), float(c)] for a, c in rows],
    }

    # ---- tol = 1e-9, doc/notebooks/Customising the adaptive integrator.ipynb
    cs = cells(os.path.join(nbdir, "Customising the adaptive integrator.ipynb"))
    out = find(cs, "ta.propagate_until(t=10.0)\nta.propagate_until(t=0.0)")
    pins["pendulum_tol1e-9"] = {
        "tol": 1e-9,
        "order": int(re.search(r"Taylor order\s*:\s*(\d+)", cs[1][1]).group(1)),
        "state_after_10_and_back": nums(re.search(r"State\s*: \[(.*?)\]", out).group(1)),
    }

    # ---- forced damped pendulum batch, doc/notebooks/Batch mode overview.ipynb
    cs = cells(os.path.join(nbdir, "Batch mode overview.ipynb"))
    q = pins["forced_pendulum_batch"] = {
        "sys": "x' = v, v' = cos(t) - par[0] * v - sin(x)",
        "state": [[0.00, 0.01, 0.02, 0.03], [1.85, 1.86, 1.87, 1.88]],
        "pars": [[0.10, 0.11, 0.12, 0.13]],
    }
    out = find(cs, "ta.step()\n\n# Print the outcomes to screen.")
    q["step_h"] = [float(x) for x in re.findall(r"-4294967297>, (" + NUM + r")\)", out)]
    out = find(cs, "ta.step([0.010, 0.011, 0.012, 0.013])")
    st = re.search(r"State:\n\[\[(.*?)\]\n \[(.*?)\]\]\nTime:\n\[(.*?)\]", out, re.S)
    q["after_clamped_step"] = {"state_8digits": [nums(st.group(1)), nums(st.group(2))], "time_8digits": nums(st.group(3))}

    def pres(s):
        return [
            {"min_h": float(a), "max_h": float(b), "n_steps": int(c)}
            for a, b, c in re.findall(r"-4294967299>,\s*(" + NUM + r"),\s*(" + NUM + r"),\s*(\d+)\)", s)
        ]

    out = find(cs, "ta.propagate_for([10.0, 11.0, 12.0, 13.0])")
    parts = out.split("Outcomes:")
    q["for"] = {"delta_t": [10.0, 11.0, 12.0, 13.0], "res": pres(parts[1])}
    q["until"] = {"t": [20.0, 21.0, 22.0, 23.0], "res": pres(parts[2])}
    for key, part in (("for", parts[1]), ("until", parts[2])):
        st = re.search(r"State:\n\[\[(.*?)\]\n \[(.*?)\]\]", part, re.S)
        q[key]["state_8digits"] = [nums(st.group(1)), nums(st.group(2))]
    out = find(cs, "ta.propagate_res", exact=True)
    q["grid"] = {"grid": "linspace(0, 100, 1000) per lane", "res": pres(out)}
    out = find(cs, "ta.update_d_output([0.01, 0.02, 0.03, 0.04])")
    q["d_output_8digits"] = [nums(r) for r in re.findall(r"\[([^\[\]]+)\]", out)]
    out = find(cs, "c_out([0.01, 0.02, 0.03, 0.04])")
    q["c_output"] = {
        "t": [10.0, 10.1, 10.2, 10.3],
        "at_0.01..0.04_8digits": [nums(r) for r in re.findall(r"\[([^\[\]]+)\]", out)],
        "c_arr_0_1_2": float(find(cs, "c_arr[0, 1, 2]", exact=True).strip()),
    }
    out = find(cs, "ta.tc[:, 0, :]", exact=True)
    q["tc_order0"] = [nums(r) for r in re.findall(r"\[([^\[\]]+)\]", out)]

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "notebook_pins.json")
    with open(path, "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/heyoka.py")
    main(sys.argv[1])
