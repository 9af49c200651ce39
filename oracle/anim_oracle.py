"""Animation oracle (test infrastructure only; never on a product path).

A numpy (float64) restatement of how the reference poses a glTF scene each
frame, from the document's JSON and binary buffer:

* channel sampling (src/renderer.cpp:1079-1149): time wraps modulo the
  channel's last key time; the previous key is the one before the first key
  later than t; STEP holds it, LINEAR mixes translations and scales and
  slerps rotations (shortest arc, linear when nearly parallel);
* node world matrices (updateWorldMatrix, src/renderer.cpp:1028-1058):
  T * R * S unless the node has a matrix, world = parent * local;
* vertices (src/renderer.cpp:1155-1230): world * (sum_k w_k * joint_k) * p
  with joint_k = inverse(world(mesh node)) * world(joint) * inverseBind,
  normals through the inverse transpose of the mesh node's world matrix.
The library differs deliberately before the first key and at the last key
(it holds the end values) and for CUBICSPLINE (it follows the glTF spline);
the fixtures exercise those cases with the library's rule, restated here.
Animation 2 is used when the document has three or more, else 0
(src/gltf_loader.cpp:1398-1400).
"""
import numpy as np

COMPS = {"translation": 3, "rotation": 4, "scale": 3}


def _accessor(doc, binary, i):
    acc = doc["accessors"][i]
    view = doc["bufferViews"][acc["bufferView"]]
    n = {"SCALAR": 1, "VEC3": 3, "VEC4": 4, "MAT4": 16, "VEC2": 2}[acc["type"]]
    dt = {5126: "<f4", 5123: "<u2", 5121: "u1", 5125: "<u4"}[acc["componentType"]]
    off = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
    a = np.frombuffer(binary, dt, acc["count"] * n, off).reshape(acc["count"], n)
    return a.astype(np.float64)


def quat_matrix(q):
    x, y, z, w = q
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                 [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                 [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]]
    return m


def slerp(a, b, t):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    c = float(a @ b)
    if c < 0:
        b, c = -b, -c
    if c > 1 - 1.1920929e-07:
        return a * (1 - t) + b * t
    ang = np.arccos(c)
    return (np.sin((1 - t) * ang) * a + np.sin(t * ang) * b) / np.sin(ang)


def sample(times, values, interp, path, t):
    """values: (keys, comps) or (3 * keys, comps) for CUBICSPLINE."""
    n = len(times)
    tmax = times[-1]
    if tmax > 0 and t > tmax:
        t = np.modf(t / tmax)[0] * tmax
    nxt = next((i for i in range(n) if times[i] > t), n)
    key = (lambda i: values[3 * i + 1]) if interp == "CUBICSPLINE" else (lambda i: values[i])
    if nxt == 0 or nxt == n or interp == "STEP":
        return key(0 if nxt == 0 else n - 1 if nxt == n else nxt - 1)
    p = nxt - 1
    td = times[nxt] - times[p]
    a = (t - times[p]) / td
    if interp == "CUBICSPLINE":
        v0, b0 = values[3 * p + 1], values[3 * p + 2]
        v1, a1 = values[3 * nxt + 1], values[3 * nxt]
        r = ((2 * a ** 3 - 3 * a ** 2 + 1) * v0 + td * (a ** 3 - 2 * a ** 2 + a) * b0 +
             (-2 * a ** 3 + 3 * a ** 2) * v1 + td * (a ** 3 - a ** 2) * a1)
        return r / np.linalg.norm(r) if path == "rotation" else r
    if path == "rotation":
        return slerp(key(p), key(nxt), a)
    return key(p) * (1 - a) + key(nxt) * a


def pose(doc, binary, t):
    """World matrix of every node at time t (4x4 float64, row-major math)."""
    nodes = doc["nodes"]
    trs = [dict(t=np.array(n.get("translation", [0, 0, 0]), np.float64),
                r=np.array(n.get("rotation", [0, 0, 0, 1]), np.float64),
                s=np.array(n.get("scale", [1, 1, 1]), np.float64)) for n in nodes]
    anims = doc.get("animations", [])
    if anims:
        an = anims[2 if len(anims) >= 3 else 0]
        for ch in an["channels"]:
            path = ch["target"]["path"]
            if path not in COMPS:
                continue
            smp = an["samplers"][ch["sampler"]]
            times = _accessor(doc, binary, smp["input"])[:, 0]
            vals = _accessor(doc, binary, smp["output"])
            v = sample(times, vals, smp.get("interpolation", "LINEAR"), path, t)
            trs[ch["target"]["node"]][path[0]] = v
    world = [None] * len(nodes)

    def local(i):
        if "matrix" in nodes[i]:
            return np.array(nodes[i]["matrix"], np.float64).reshape(4, 4).T
        T = np.eye(4)
        T[:3, 3] = trs[i]["t"]
        S = np.diag(list(trs[i]["s"]) + [1.0])
        return T @ quat_matrix(trs[i]["r"]) @ S

    def walk(i, parent):
        world[i] = parent @ local(i)
        for c in nodes[i].get("children", []):
            walk(c, world[i])

    for r in doc["scenes"][doc["scene"]]["nodes"]:
        walk(r, np.eye(4))
    return world


def vertices(doc, binary, t):
    """World positions and normals of every vertex, in the order the library
    flattens them (scene nodes depth first, primitives in order, indexed
    primitives keep their vertex order)."""
    world = pose(doc, binary, t)
    P, N = [], []

    def walk(i):
        node = doc["nodes"][i]
        if "mesh" in node:
            G = world[i]
            nm = np.linalg.inv(G[:3, :3]).T
            joints = None
            if "skin" in node:
                sk = doc["skins"][node["skin"]]
                ibm = _accessor(doc, binary, sk["inverseBindMatrices"]).reshape(-1, 4, 4).transpose(0, 2, 1)
                inv = np.linalg.inv(G)
                joints = [inv @ world[j] @ ibm[k] for k, j in enumerate(sk["joints"])]
            for pr in doc["meshes"][node["mesh"]]["primitives"]:
                at = pr["attributes"]
                p = _accessor(doc, binary, at["POSITION"])
                n = _accessor(doc, binary, at["NORMAL"]) if "NORMAL" in at else np.zeros_like(p)
                if joints is not None and "JOINTS_0" in at:
                    jj = _accessor(doc, binary, at["JOINTS_0"]).astype(int)
                    ww = _accessor(doc, binary, at["WEIGHTS_0"])
                    for v in range(len(p)):
                        S = sum(ww[v, k] * joints[jj[v, k]] for k in range(4))
                        P.append((G @ S @ np.r_[p[v], 1.0])[:3])
                else:
                    P.extend((G @ np.c_[p, np.ones(len(p))].T).T[:, :3])
                N.extend((nm @ n.T).T)
        for c in node.get("children", []):
            walk(c)

    for r in doc["scenes"][doc["scene"]]["nodes"]:
        walk(r)
    return np.array(P), np.array(N)
