"""Minimal Bio.Phylo stand-in (test-only): Newick reading and writing."""

import io

from . import BaseTree


def _tokenize(text):
    i, n = 0, len(text)
    while i < n:
        ch = text[i]
        if ch in "(),:;":
            yield ch
            i += 1
        elif ch == "[":
            i = text.index("]", i) + 1
        elif ch.isspace():
            i += 1
        elif ch == "'":
            j = text.index("'", i + 1)
            yield ("label", text[i + 1:j])
            i = j + 1
        else:
            j = i
            while j < n and text[j] not in "(),:;[" and not text[j].isspace():
                j += 1
            yield ("label", text[i:j])
            i = j


def _is_number(s):
    try:
        float(s)
        return True
    except ValueError:
        return False


def _parse_newick(text):
    root = BaseTree.Clade()
    stack = [root]
    current = root
    expect_length = False
    after_close = False
    for tok in _tokenize(text):
        if tok == "(":
            child = BaseTree.Clade()
            current.clades.append(child)
            stack.append(current)
            current = child
            after_close = False
        elif tok == ",":
            parent = stack[-1]
            child = BaseTree.Clade()
            parent.clades.append(child)
            current = child
            after_close = False
        elif tok == ")":
            current = stack.pop()
            after_close = True
        elif tok == ":":
            expect_length = True
        elif tok == ";":
            break
        else:
            value = tok[1]
            if expect_length:
                current.branch_length = float(value)
                expect_length = False
            elif after_close and _is_number(value):
                current.confidence = float(value)
            else:
                current.name = value
    return BaseTree.Tree(root=root, rooted=False)


def read(file, format):
    if format not in ("newick", "nwk"):
        raise ValueError("bioshim Phylo.read supports newick only")
    if hasattr(file, "read"):
        text = file.read()
    else:
        with open(file) as fh:
            text = fh.read()
    return _parse_newick(text)


def _write_clade(c):
    s = ""
    if c.clades:
        s = "(" + ",".join(_write_clade(ch) for ch in c.clades) + ")"
    if c.name:
        s += c.name
    if c.branch_length is not None:
        s += ":%r" % float(c.branch_length)
    return s


def write(tree, file, format):
    text = _write_clade(tree.root) + ";\n"
    if hasattr(file, "write"):
        file.write(text)
    else:
        with open(file, "w") as fh:
            fh.write(text)
    return 1


def parse(file, format):
    yield read(file, format)


__all__ = ["BaseTree", "read", "write", "parse", "io"]
