"""Insertion of space-charge nodes into a lattice
(py/orbit/space_charge/scLatticeModifications.py:10-61)."""
from orbit.lattice import AccNode


def setSC_General_AccNodes(lattice, sc_path_length_min, space_charge_calculator, SC_NodeConstructor):
    """Walks all parts of the first-level nodes; a node is placed at the start
    of a part once the path since the previous node exceeds
    sc_path_length_min, as a BODY/BEFORE child.  Each node's kick length is
    the path to the next node; the first node (at the lattice start) covers
    the rest of the lattice.  Returns the list of SC nodes."""
    accNodes = lattice.getNodes()
    if len(accNodes) == 0:
        return
    nodes_arr = []
    length_total = 0.0
    running_path = 0.0
    for accNode in accNodes:
        for ip in range(accNode.getnParts()):
            part_length = accNode.getLength(ip)
            if part_length > 1.0:
                print("Warning! Node ", accNode.getName(), " has length ", part_length,
                      "m which is great than 1 m.  Space charge algorithm may be innacurate!")
            if running_path > sc_path_length_min:
                nodes_arr.append((accNode, ip, length_total, running_path))
                running_path = 0.0
            running_path += part_length
            length_total += part_length
    if len(nodes_arr) > 0:
        rest_length = length_total - nodes_arr[len(nodes_arr) - 1][2]
    else:
        rest_length = length_total
    nodes_arr.insert(0, (accNodes[0], 0, 0.0, rest_length))
    scNodes_arr = []
    for inode in range(len(nodes_arr) - 1):
        (accNode, part_index, position, path_length) = nodes_arr[inode]
        (_, _, _, path_lengthNext) = nodes_arr[inode + 1]
        scNode = SC_NodeConstructor(space_charge_calculator, accNode.getName() + ":" + str(part_index) + ":")
        scNode.setLengthOfSC(path_lengthNext)
        scNodes_arr.append(scNode)
        accNode.addChildNode(scNode, AccNode.BODY, part_index, AccNode.BEFORE)
    (accNode, part_index, position, path_length) = nodes_arr[len(nodes_arr) - 1]
    scNode = SC_NodeConstructor(space_charge_calculator, accNode.getName() + ":" + str(part_index) + ":")
    scNode.setLengthOfSC(rest_length)
    scNodes_arr.append(scNode)
    accNode.addChildNode(scNode, AccNode.BODY, part_index, AccNode.BEFORE)
    return scNodes_arr
