"""Train the learned SGS correction on the 32^3 case and store it as a test fixture.

    python tests/golden/make_sgs_net.py OUT.npz        (on a GB300; about 3 minutes)

Runs lex_gb300.learned_sgs.experiment() with its defaults (seeded 100 m warm-bubble runs
coarse-grained to 600 m x 600 m x 300 m; an a-priori stage, then training through the solver from
the a-priori weights and from an untrained network; the branch and iteration with the best
validation score are kept) and writes the chosen network's weights, the input/output ranges of
the packing (lo, rin per level; the output range per level, which the training uses at every
point of the level) and the run's summary.  tests/test_gpu_learned_sgs.py evaluates the stored
network on the held-out run against Smagorinsky alone.
"""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))


def main(out):
    from lex_gb300 import learned_sgs as L
    r = L.experiment()
    net, scale = r.pop("net"), r.pop("scale")
    sd = net.state_dict()
    arrays = {"w%d" % i: t.detach().numpy() for i, t in enumerate(sd["w"])}
    arrays.update({"b%d" % i: t.detach().numpy() for i, t in enumerate(sd["b"])})
    arrays["lo"] = scale["lo"].detach().cpu().numpy()
    arrays["rin"] = scale["rin"].detach().cpu().numpy()
    arrays["rout_level"] = scale["rout"][:, :, 0, 0].detach().cpu().numpy()
    arrays["summary"] = np.asarray(json.dumps(r))
    np.savez_compressed(out, **arrays)
    print(json.dumps({k: r[k] for k in ("chosen", "theta_err_smagorinsky", "theta_err_learned", "cost_ratio")}))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_sgs_net.py OUT.npz")
    main(sys.argv[1])
