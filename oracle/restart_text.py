"""ORACLE -- test infrastructure only.

Pure-Python restatement of the reference's restart file text (the oracle
for gbfv_format_restart / gbfv_parse_restart).  Only tests/ may import it.
Parity status: unpinned against files written by the reference (it cannot
be built here); the layout follows the reference's source text:

  Restart::serializeBegin / serializeSectionBegin / serializeSectionEnd /
  serializeEntities       opm/models/io/restart.hh:57-75, 101-160
  Simulator::serialize    opm/models/utils/simulator.hh:906-943
  FvBaseProblem::serialize -> VtkMultiWriter::serialize
                          fvbaseproblem.hh:755-760, vtkmultiwriter.hh:408-437
  EcfvDiscretization::serialize (codim 0)
                          ecfvdiscretization.hh:212-213
  VcfvDiscretization::serialize (codim dim: the vertices)
                          vcfvdiscretization.hh:185-200
  FvBaseDiscretization::serializeEntity
                          fvbasediscretization.hh:1440-1454
  BlackOilModel::serializeEntity
                          blackoilmodel.hh:468-493

The stream has precision(20) (restart.hh:115): a double is written as
"%.20g", an integer plainly.
"""


def _g(x):
    return "%.20g" % x


def cookie(num_cpus, rank, num_elements, num_edges, num_vertices):
    """restart.hh:57-75 (gridName is the fixed string 'blubb')."""
    return ("eWoms restart file: gridName='blubb' numCPUs=%d myRank=%d numElements=%d numEdges=%d "
            "numVertices=%d" % (num_cpus, rank, num_elements, num_edges, num_vertices))


def format_restart(pv, gas_meaning=None, *, num_edges, num_vertices, num_cpus=1, rank=0, episode_index=0,
                   episode_start_time=0.0, episode_length=0.0, start_time=0.0, time=0.0, time_step_index=0,
                   vtk_section=True, vtk_writer_num=0, entity_codim=0, num_elements=None):
    """Text of the restart file of primary variables pv (num_cells x b,
    natural cell order); gas_meaning (black-oil) adds the meanings and the
    PVT region after the variables (water Sw = 0, pressure Po = 0, region 0).
    entity_codim > 0: the entities are a vertex-centred grid's vertices and
    num_elements its element count (the cookie's numElements)."""
    out = []
    # serializeBegin: the cookie section (no content)
    ne = len(pv) if entity_codim == 0 else num_elements
    out.append(cookie(num_cpus, rank, ne, num_edges, num_vertices) + "\n")
    out.append("\n")
    # Simulator section: six values, each followed by a blank, then the end
    out.append("Simulator\n")
    out.append("%d %s %s %s %s %d " % (episode_index, _g(episode_start_time), _g(episode_length),
                                       _g(start_time), _g(time), time_step_index))
    out.append("\n")
    if vtk_section:
        # writer count, then meta-file length and position (no meta file here)
        out.append("VTKMultiWriter\n")
        out.append("%d\n" % vtk_writer_num)
        out.append("0  0\n")
        out.append("\n")
    out.append("Entities: Codim %d\n" % entity_codim)
    for c, row in enumerate(pv):
        line = "".join(_g(v) + " " for v in row)
        if gas_meaning is not None:
            line += "%d 0 0 0 " % int(gas_meaning[c])
        out.append(line + "\n")
    out.append("\n")
    return "".join(out).encode()


def file_name(output_dir, sim_name, time, rank=0):
    """Restart::restartFileName_ (restart.hh:80-95): the time as an ostream
    writes it by default ("%g")."""
    d = output_dir or ""
    if d == ".":
        d = ""
    elif d and not d.endswith("/"):
        d += "/"
    return "%s%s_time=%s_rank=%d.ers" % (d, sim_name, "%g" % time, rank)
