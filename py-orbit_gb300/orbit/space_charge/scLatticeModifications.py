"""Insertion of space-charge nodes into a lattice
(py/orbit/space_charge/scLatticeModifications.py:10-61)."""
from orbit.lattice import AccNode


def setSC_General_AccNodes(lattice, sc_path_length_min, space_charge_calculator, SC_NodeConstructor):
    """Places SC nodes as BODY/BEFORE children of the first-level nodes and
    returns them in lattice order.

    The rule (which decides the maps between kicks, so it is kept exactly):
    the parts of the first-level nodes are walked in order; a part that
    starts once the path walked since the previous placement exceeds
    sc_path_length_min gets a node.  One more node sits at the start of the
    lattice.  Each node kicks for the path up to the next node (the path
    summed part by part since that placement), the last one for the path
    from its position to the end of the lattice.  Parts longer than 1 m get
    a warning.  Nodes are named "<node name>:<part index>:"."""
    nodes = lattice.getNodes()
    if len(nodes) == 0:
        return
    # placements found by the walk: (node, part index, path from the lattice
    # start to the part, path walked since the previous placement)
    found = []
    since_previous = 0.0
    walked = 0.0
    for node in nodes:
        for part in range(node.getnParts()):
            part_length = node.getLength(part)
            if part_length > 1.0:
                print("Warning: part %d of node %s is %s m long (more than 1 m); the space-charge kicks may be "
                      "inaccurate" % (part, node.getName(), part_length))
            if since_previous > sc_path_length_min:
                found.append((node, part, walked, since_previous))
                since_previous = 0.0
            since_previous += part_length
            walked += part_length
    last_position = found[-1][2] if found else 0.0
    placements = [(nodes[0], 0)] + [(node, part) for node, part, _, _ in found]
    kick_lengths = [path for _, _, _, path in found] + [walked - last_position]
    sc_nodes = []
    for (node, part), kick_length in zip(placements, kick_lengths):
        sc_node = SC_NodeConstructor(space_charge_calculator, node.getName() + ":" + str(part) + ":")
        sc_node.setLengthOfSC(kick_length)
        node.addChildNode(sc_node, AccNode.BODY, part, AccNode.BEFORE)
        sc_nodes.append(sc_node)
    return sc_nodes
