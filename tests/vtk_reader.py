"""Reader of the legacy binary VTK PolyData files lpm_bve_vtk_write produces (test helper)."""


def read_vtk_sections(raw):
    """Splits a legacy binary VTK PolyData file into its four header lines and a list of
    (keyword line, payload bytes) records."""
    out, pos = [], 0
    header = []
    for _ in range(4):
        end = raw.index(b"\n", pos)
        header.append(raw[pos:end].decode())
        pos = end + 1
    sizes = {"double": 8, "int": 4}
    count = 0
    while pos < len(raw):
        while pos < len(raw) and raw[pos:pos + 1] == b"\n":
            pos += 1
        if pos >= len(raw):
            break
        end = raw.index(b"\n", pos)
        line = raw[pos:end].decode()
        pos = end + 1
        parts = line.split()
        if parts[0] == "POINTS":
            n = int(parts[1]) * 3 * sizes[parts[2]]
        elif parts[0] == "POLYGONS":
            n = int(parts[2]) * 4
        elif parts[0] in ("POINT_DATA", "CELL_DATA"):
            out.append((line, b""))
            count = int(parts[1])
            continue
        elif parts[0] == "SCALARS":
            end = raw.index(b"\n", pos)  # the LOOKUP_TABLE line
            pos = end + 1
            n = count * 8
        elif parts[0] == "VECTORS":
            n = count * 3 * 8
        else:
            raise AssertionError(line)
        out.append((line, raw[pos:pos + n]))
        assert len(raw[pos:pos + n]) == n, line
        pos += n
    return header, out
