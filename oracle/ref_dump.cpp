// ref_dump — TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own construction code and writes what the -s run
// never prints: every surviving k-molecule with its 8 edge multiplicities.
// The reference's graph.cpp is compiled in through the include below (its
// main() renamed), from the reference tree given on the compiler's include
// path; nothing of it is copied here.
//
// Call sequence = the reference main() up to the node build
// (graph.cpp:3452-3561), then printLocalNodeGraph (graph.cpp:555-572) into
// <o>/nodes.txt instead of the gather/merge stages. nodes.txt lists the nodes
// in the node map's iteration order, which is the order the merge stage
// visits them (graph.cpp:1412). With -d the run continues like the
// reference's own -d run: simplifyDistNodeGraph (graph.cpp:1392-1566), then
// gatherDistNodeGraph written to <o>/contigGraph.txt (graph.cpp:3611-3621).
// Usage is the reference's own: ref_dump -k K -c C -i reads.fa -o <new dir> [-d]
#define main swap_reference_main
#include "graph.cpp"
#undef main

int main(int argc, char *argv[]) {
    MPIEnviroment MPIcontrol;
    MPIcontrol.init(argc, argv);
    parameter parameters;
    parameters.getParameters(argc, argv, &MPIcontrol);

    kmerGraph *mygraph = new kmerGraph;
    distNodeGraph *nodeGraph = new distNodeGraph(&parameters, &MPIcontrol);
    nodeGraph->constructDistNodeGraph(mygraph, &parameters, &MPIcontrol);
    delete mygraph;
    nodeGraph->cutoffGraph(&MPIcontrol, parameters.cutoffThreshold);
    nodeGraph->buildKmoleculeGraph(&MPIcontrol, &parameters);
    nodeGraph->graphStatistics(&parameters, &MPIcontrol);

    strcpy(parameters.kmerGraph, parameters.outputPath);
    strcat(parameters.kmerGraph, "/nodes.txt");
    nodeGraph->printLocalNodeGraph(&parameters, &MPIcontrol);
    if (parameters.distGraphFlag) {
        nodeGraph->simplifyDistNodeGraph(&parameters, &MPIcontrol);
        char *rBuf = nodeGraph->gatherDistNodeGraph(&parameters, &MPIcontrol);
        FILE *fp = fopen(parameters.graphPath, "w");
        fprintf(fp, "%s\n", rBuf);
        fclose(fp);
    }
    MPIcontrol.finalize();
    return 0;
}
