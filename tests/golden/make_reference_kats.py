"""Extracts the known-answer constants of the reference crate's own tests into reference_kats.json.

Run in a checkout that has the reference sources (pass their root as argv[1]); the JSON it writes is
committed so the test suite never needs the reference at run time. Every value is read from the
reference's source text, with the file and line it came from recorded beside it.
"""

import json
import os
import re
import sys


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read().split("\n")


def find_hex_const(lines, name):
    for i, line in enumerate(lines):
        if re.search(r"\b%s\b.*=.*(EngineId::new\(hex!\(|Hash\(hex!\()" % name, line):
            m = re.search(r'"([0-9a-f]{64})"', lines[i + 1]) or re.search(r'"([0-9a-f]{64})"', line)
            if m:
                return m.group(1), i + 1
    raise KeyError(name)


def challenge_index_cases(lines):
    """Parses the MockSponge tests of challenge_indices.rs into (squeeze, num_leaves, count, dedup, expected)."""
    cases = []
    i = 0
    while i < len(lines):
        if lines[i].strip().startswith("fn test_challenge_stir_queries"):
            start = i
            body = []
            depth = 0
            j = i
            while True:
                body.append(lines[j])
                depth += lines[j].count("{") - lines[j].count("}")
                j += 1
                if depth == 0 and len(body) > 1:
                    break
            text = "\n".join(re.sub(r"//.*", "", ln) for ln in body)
            num_leaves = eval(re.search(r"let num_leaves = ([^;]+);", text).group(1).replace("<<", "<<"))
            count = int(re.search(r"let num_queries = (\d+);", text).group(1))
            sq = re.search(r"squeeze: &\[(.*?)\]", text, re.S).group(1)
            squeeze = [int(x, 16) for x in re.findall(r"0x[0-9A-Fa-f]{2}", sq)]
            dedup = "true" in re.search(r"challenge_indices\(&mut prover_state, num_leaves, num_queries, (\w+)\)",
                                        text).group(1)
            env = {"num_leaves": num_leaves}
            idx_defs = re.findall(r"let index_(\d+) = ([^;]+);", text)
            if idx_defs:
                expected = [eval(expr, {}, env) for _, expr in idx_defs]
            else:
                exp = re.search(r"let mut expected_indices = vec!\[(.*?)\];", text, re.S).group(1)
                expected = [eval(e.strip(), {}, env) for e in exp.split(",") if e.strip()]
            expected = sorted(set(expected)) if dedup else expected
            cases.append({"name": lines[start].strip().split("(")[0][3:], "line": start + 1, "squeeze": squeeze,
                          "num_leaves": num_leaves, "count": count, "dedup": dedup, "expected": expected})
            i = j
        else:
            i += 1
    return cases


def struct_fields(lines, name, after=0):
    """Field names, in declaration order, of the first `struct <name>` at or after line `after`,
    with serde renames applied (the names serde writes as map keys), and the struct's line."""
    i = after
    while i < len(lines):
        if re.match(r"\s*(pub\s+)?struct\s+%s\b" % name, lines[i]) and "(" not in lines[i].split(name, 1)[1][:2]:
            break
        i += 1
    else:
        raise KeyError(name)
    start = i
    while "{" not in lines[i]:
        i += 1
    fields, rename = [], None
    i += 1
    while not lines[i].strip().startswith("}"):
        ln = lines[i].strip()
        m = re.search(r'#\[serde\(rename = "([^"]+)"\)\]', ln)
        if m:
            rename = m.group(1)
        m = re.match(r"(pub\s+)?(\w+)\s*:", ln)
        if m and not ln.startswith("//") and not ln.startswith("#"):
            fields.append(rename or m.group(2))
            rename = None
        i += 1
    return fields, start + 1


def type_info_string(lines, embedding):
    """The TypeInfo string of an embedding type (`impl ... TypeInfo for <embedding><F>`)."""
    for i, ln in enumerate(lines):
        if re.search(r"impl<.*> TypeInfo for %s<" % embedding, ln):
            for j in range(i, i + 8):
                m = re.search(r'"(\w+)"\.into\(\)', lines[j])
                if m:
                    return m.group(1), j + 1
    raise KeyError(embedding)


def serde_layout(root):
    """Field names and order of every serde struct in whir::Config's serialized form (the CBOR map
    keys ciborium writes for the protocol id), with the file:line of each struct."""
    specs = [("whir_config", "src/protocols/whir/mod.rs", "Config"),
             ("round_config", "src/protocols/whir/mod.rs", "RoundConfig"),
             ("irs_config", "src/protocols/irs_commit.rs", "Config"),
             ("matrix_config", "src/protocols/matrix_commit.rs", "Config"),
             ("merkle_config", "src/protocols/merkle_tree.rs", "Config"),
             ("merkle_layer", "src/protocols/merkle_tree.rs", "LayerConfig"),
             ("sumcheck_config", "src/protocols/sumcheck.rs", "Config"),
             ("pow_config", "src/protocols/proof_of_work.rs", "Config"),
             ("field_info", "src/algebra/fields.rs", "FieldInfo"),
             ("identity", "src/algebra/embedding.rs", "Identity"),
             ("basefield", "src/algebra/embedding.rs", "Basefield"),
             ("typed_value", "src/type_info.rs", "TypedValue")]
    out = {}
    for key, rel, name in specs:
        fields, line = struct_fields(read(root, rel), name)
        out[key] = {"fields": fields, "at": "%s:%d" % (rel, line)}
    emb = read(root, "src/algebra/embedding.rs")
    for e in ("Identity", "Basefield"):
        s, line = type_info_string(emb, e)
        out[e.lower() + "_type_info"] = {"value": s, "at": "src/algebra/embedding.rs:%d" % line}
    return out


def main(root):
    out = {"source": "WizardOfMenlo/whir reference sources"}
    b3 = read(root, "src/hash/blake3_engine.rs")
    dg = read(root, "src/hash/digest_engine.rs")
    cp = read(root, "src/hash/copy_engine.rs")
    ids = {}
    for name, lines, rel in (("BLAKE3", b3, "src/hash/blake3_engine.rs"), ("SHA2", dg, "src/hash/digest_engine.rs"),
                             ("SHA3", dg, "src/hash/digest_engine.rs"), ("KECCAK", dg, "src/hash/digest_engine.rs"),
                             ("COPY", cp, "src/hash/copy_engine.rs")):
        h, line = find_hex_const(lines, name)
        ids[name] = {"hex": h, "at": "%s:%d" % (rel, line)}
    out["engine_ids"] = ids
    # Engine id preimages: SHA3-256("whir::hash" || oid bytes or name) (src/hash/mod.rs:88-103)
    out["engine_id_preimages"] = {
        "BLAKE3": {"name": "Blake3"}, "COPY": {"name": "copy"}, "KECCAK": {"name": "keccak"},
        "SHA2": {"oid_der_body": "608648016503040201"}, "SHA3": {"oid_der_body": "608648016503040208"},
    }
    h, line = find_hex_const(b3, "EMPTY_HASH")
    out["blake3_empty_hash"] = {"hex": h, "at": "src/hash/blake3_engine.rs:%d" % line}
    ci = read(root, "src/protocols/challenge_indices.rs")
    out["challenge_indices"] = challenge_index_cases(ci)
    # PoW threshold / difficulty KATs (proof_of_work.rs test_threshold_integer / test_difficulty_integer)
    pw = "\n".join(read(root, "src/protocols/proof_of_work.rs"))
    assert "threshold(Bits::new(0.0)), u64::MAX" in pw and "threshold(Bits::new(60.0)), 1 << 4" in pw
    assert "threshold(Bits::new(bits as f64)), 1 << (64 - bits)" in pw
    out["pow_threshold"] = [[0.0, 2**64 - 1], [60.0, 1 << 4]] + [[float(b), 1 << (64 - b)] for b in range(1, 61)]
    out["pow_difficulty"] = [[2**64 - 1, 0.0], [1 << 4, 60.0]] + [[1 << (64 - b), float(b)] for b in range(1, 61)]
    mt = read(root, "src/protocols/merkle_tree.rs")
    table = []
    for line in mt:
        m = re.search(r"assert_eq!\(layers_for_size\((\d+)\), (\d+)\);", line)
        if m:
            table.append([int(m.group(1)), int(m.group(2))])
    out["layers_for_size"] = table
    ct = "\n".join(read(root, "src/algebra/ntt/cooley_tukey.rs"))
    assert "assert_eq!(engine.order, 3 << 32);" in ct
    out["goldilocks"] = {"modulus": 18446744069414584321, "generator": 7, "engine_order": 3 << 32,
                         "at": "src/algebra/fields.rs:85-91, src/algebra/ntt/cooley_tukey.rs:583-595"}
    fl = "\n".join(read(root, "src/algebra/fields.rs"))
    m = re.search(r'"\{\\"characteristic\\":\\"([0-9a-f]+)\\",\\"extension_degree\\":(\d+)\}"', fl)
    out["field_type_info_goldilocks3"] = {"characteristic": m.group(1), "extension_degree": int(m.group(2))}
    out["serde_config_layout"] = serde_layout(root)
    tw = "\n".join(read(root, "src/algebra/ntt/cooley_tukey.rs"))
    assert "assert_eq!(values[4], Field64::from(5) * roots[10]);" in tw
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_kats.py <root of the reference crate's sources>")
    data = main(sys.argv[1])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", path)
